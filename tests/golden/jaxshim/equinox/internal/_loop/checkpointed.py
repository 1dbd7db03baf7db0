def checkpointed_while_loop(cond_fun, body_fun, init_val, *, max_steps=None, checkpoints=None, **_):
    """A plain while loop: checkpointing changes only what reverse mode stores."""
    val = init_val
    steps = 0
    while bool(cond_fun(val)):
        if max_steps is not None and steps >= max_steps:
            break
        val = body_fun(val)
        steps += 1
    return val
