"""Keys are paths; the golden script registers the draw each key must return."""
import torch

DRAWS = {}


class Key:
    def __init__(self, path):
        self.path = path

    def __repr__(self):
        return f"Key({self.path})"


def PRNGKey(seed):
    return Key(str(seed))


def split(key, num=2):
    return [Key(f"{key.path}.{i}") for i in range(num)]


def _draw(key, shape):
    if key.path not in DRAWS:
        raise KeyError(f"no scripted draw for key {key.path}")
    v = torch.as_tensor(DRAWS[key.path], dtype=torch.float64)
    if tuple(shape) and tuple(v.shape) != tuple(shape):
        raise ValueError(f"scripted draw for {key.path} has shape {tuple(v.shape)}, wanted {tuple(shape)}")
    return v


def normal(key, shape=(), dtype=None):
    return _draw(key, shape)


def uniform(key, shape=(), dtype=None, minval=0.0, maxval=1.0):
    return _draw(key, shape)


def choice(key, a, shape=(), replace=True, p=None):
    """The scripted indices into a (with replacement)."""
    idx = torch.as_tensor(DRAWS[key.path], dtype=torch.long)
    return torch.as_tensor(a)[idx]


def multivariate_normal(key, mean, cov, shape=(), dtype=None):
    """mean + z @ cholesky(cov).T with the scripted standard normals z
    (jax.random.multivariate_normal's default Cholesky method)."""
    mean = torch.as_tensor(mean, dtype=torch.float64)
    cov = torch.as_tensor(cov, dtype=torch.float64)
    z = _draw(key, tuple(shape) + (mean.shape[-1],))
    return mean + z @ torch.linalg.cholesky(cov).T
