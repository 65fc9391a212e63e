import dataclasses


def field(pytree_node=True, **kwargs):
    return dataclasses.field(**kwargs)


def dataclass(cls=None, **kw):
    def wrap(c):
        d = dataclasses.dataclass(frozen=True)(c)
        d.replace = lambda self, **changes: dataclasses.replace(self, **changes)
        return d
    return wrap if cls is None else wrap(cls)
