import torch


def inv(a):
    a = torch.as_tensor(a, dtype=torch.float64)
    return torch.linalg.inv(a) if a.dim() == 2 else 1.0 / a


def cholesky(a):
    a = torch.as_tensor(a, dtype=torch.float64)
    return torch.linalg.cholesky(a) if a.dim() == 2 else torch.sqrt(a)
