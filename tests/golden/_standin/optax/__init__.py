"""optax stand-in: annotation names, plus adam / chain / apply_updates /
projections.projection_box for the golden-fixture script (Kingma & Ba's Adam
with optax's defaults: b1 0.9, b2 0.999, eps 1e-8, eps_root 0, bias
correction 1 - b**t, update scaled by -learning_rate)."""
import types

import torch


class GradientTransformation:
    pass


class OptState:
    pass


class _Adam:
    def __init__(self, learning_rate, b1=0.9, b2=0.999, eps=1e-8, eps_root=0.0):
        self.lr, self.b1, self.b2, self.eps, self.eps_root = learning_rate, b1, b2, eps, eps_root

    def init(self, params):
        p = torch.as_tensor(params, dtype=torch.float64)
        return (0, torch.zeros_like(p), torch.zeros_like(p))

    def update(self, g, state, params=None):
        count, mu, nu = state
        mu = (1 - self.b1) * g + self.b1 * mu
        nu = (1 - self.b2) * g * g + self.b2 * nu
        c = count + 1
        mu_hat = mu / (1 - self.b1 ** c)
        nu_hat = nu / (1 - self.b2 ** c)
        return -self.lr * (mu_hat / (torch.sqrt(nu_hat + self.eps_root) + self.eps)), (c, mu, nu)


def adam(learning_rate, b1=0.9, b2=0.999, eps=1e-8, eps_root=0.0):
    return _Adam(learning_rate, b1, b2, eps, eps_root)


def chain(*transforms):
    if len(transforms) != 1:
        raise NotImplementedError("the stand-in chains a single transformation")
    return transforms[0]


def apply_updates(params, updates):
    return params + updates


def _projection_box(x, lower, upper):
    return torch.minimum(torch.maximum(x, torch.as_tensor(lower, dtype=x.dtype)), torch.as_tensor(upper, dtype=x.dtype))


projections = types.SimpleNamespace(projection_box=_projection_box)


def __getattr__(name):
    raise NotImplementedError(f"optax.{name} is not available in the golden-fixture stand-in")
