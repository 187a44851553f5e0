"""optax stand-in: names used in annotations only."""


class GradientTransformation:
    pass


class OptState:
    pass


def __getattr__(name):
    raise NotImplementedError(f"optax.{name} is not available in the golden-fixture stand-in")
