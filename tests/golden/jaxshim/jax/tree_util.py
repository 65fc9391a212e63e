def tree_map(f, *trees):
    return f(*trees)


def tree_flatten(t):
    return [t], None


def tree_unflatten(d, leaves):
    return leaves[0]


def register_pytree_node(*a, **k):
    return None
