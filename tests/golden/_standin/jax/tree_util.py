import functools

Partial = functools.partial


def register_pytree_node_class(cls):
    return cls
