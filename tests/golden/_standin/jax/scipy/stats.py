import math

import torch


class _MVN:
    @staticmethod
    def logpdf(x, mean, cov):
        """Multivariate normal log-density; cov a scalar (isotropic) or a matrix."""
        x = torch.as_tensor(x, dtype=torch.float64)
        mean = torch.as_tensor(mean, dtype=torch.float64)
        cov_t = torch.as_tensor(cov, dtype=torch.float64)
        if cov_t.dim() == 2:
            y = x - mean
            sol = torch.linalg.solve(cov_t, y.unsqueeze(-1)).squeeze(-1)
            n = y.shape[-1]
            return -0.5 * (y * sol).sum(-1) - 0.5 * (n * math.log(2 * math.pi) + torch.logdet(cov_t))
        if cov_t.dim() != 0:
            raise NotImplementedError("covariance of rank 1")
        y = x - mean
        n = y.shape[-1]
        return -0.5 * (y * y).sum(-1) / cov_t - 0.5 * n * (math.log(2 * math.pi) + torch.log(cov_t))


multivariate_normal = _MVN()
