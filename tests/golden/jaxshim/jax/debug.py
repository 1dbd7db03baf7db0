def callback(fun, *args, **kwargs):
    kwargs.pop("ordered", None)
    fun(*args, **kwargs)


def print(fmt, *args, **kwargs):  # noqa: A001
    import builtins
    builtins.print(fmt.format(*args, **kwargs))
