"""jaxtyping stand-in: subscriptable placeholders for annotations."""


class _Ann:
    def __class_getitem__(cls, item):
        return cls


class Array(_Ann):
    pass


class Float(_Ann):
    pass


class Int(_Ann):
    pass


class Bool(_Ann):
    pass


class PRNGKeyArray(_Ann):
    pass


class PyTree(_Ann):
    pass
