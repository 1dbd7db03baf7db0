def beartype(fun=None, **_):
    if fun is None:
        return lambda f: f
    return fun
