import math

import torch


class _MVN:
    @staticmethod
    def logpdf(x, mean, cov):
        """Isotropic normal when cov is a scalar (the form the reference's MALA uses)."""
        x = torch.as_tensor(x, dtype=torch.float64)
        mean = torch.as_tensor(mean, dtype=torch.float64)
        cov_t = torch.as_tensor(cov, dtype=torch.float64)
        if cov_t.dim() != 0:
            raise NotImplementedError("matrix covariance")
        y = x - mean
        n = y.shape[-1]
        return -0.5 * (y * y).sum(-1) / cov_t - 0.5 * n * (math.log(2 * math.pi) + torch.log(cov_t))


multivariate_normal = _MVN()
