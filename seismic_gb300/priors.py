"""Priors of the Bayesian inversion, generalised from the reference's fixed 70x70 grid.

Restates jcottaar/seismic ``core/seis_prior.py`` on torch FP64 tensors of the
engine's device, for any model grid nz x nx (the reference hard-codes 70x70 and
4901 unknowns, ``core/seis_prior.py:34-35,41-42``).  A prior supplies a basis B
(model vector = B x, the last basis vector carrying min_vel), a penalty
``lambda * cost(x)`` and its gradient; ``cost_and_gradient`` combines it with
the seismogram misfit.

| class | reference |
|---|---|
| Prior | ``Prior`` core/seis_prior.py:17-64 |
| RowTotalVariation | core/seis_prior.py:67-108 |
| TotalVariation | core/seis_prior.py:112-176 |
| SquaredExponential | core/seis_prior.py:181-241 |
| RestrictFlatAreas | core/seis_prior.py:244-280 (+ label_thresholded_components, core/seis_numerics.py:81-124) |
"""
from __future__ import annotations

import math

import numpy as np
import torch

F64 = torch.float64


def _dev(device):
    return torch.device(device) if device is not None else torch.device("cuda")


class IdentityBasis:
    """The identity basis as an operator (the reference stores a sparse identity,
    core/seis_prior.py:132,227): ``B @ x`` and ``B.T @ g`` return their argument, so no
    nv x nv matrix is ever formed (175001^2 doubles for a 350x500 model)."""

    def __init__(self, n: int, device):
        self.n = n
        self.device = device
        self.shape = (n, n)

    @property
    def T(self):  # noqa: N802
        return self

    def __matmul__(self, x):
        assert x.shape[0] == self.n
        return x

    def dense(self) -> torch.Tensor:
        return torch.eye(self.n, dtype=F64, device=self.device)


class Prior:
    """Base: ``N`` unknowns, weight ``lam`` (the reference's lambda), basis (nv x N)."""

    def __init__(self, nz: int = 70, nx: int = 70, device=None):
        self.nz, self.nx = nz, nx
        self.nv = nz * nx + 1
        self.N = -1
        self.lam = 1.0
        self.prepped = False
        self.basis_vectors = None
        self.device = _dev(device)

    # core/seis_prior.py:28-45
    def prep(self):
        if not self.prepped:
            self._prep()
        self.prepped = True
        assert self.basis_vectors.shape == (self.nv, self.N)
        return self

    def adapt(self, velocity_guess):
        assert self.prepped
        self._adapt(velocity_guess)
        assert self.basis_vectors.shape == (self.nv, self.N)

    def _adapt(self, velocity_guess):
        pass

    def _identity_basis(self):
        return IdentityBasis(self.nv, self.device)

    def same_settings(self, other) -> bool:
        """True when ``other`` computes the same penalty (shared basis and weights)."""
        return (self.nz, self.nx, self.N, self.lam) == (other.nz, other.nx, other.N, other.lam) and \
            getattr(self, "epsilon", None) == getattr(other, "epsilon", None)

    # core/seis_prior.py:47-64
    def compute_cost_and_gradient(self, x: torch.Tensor, compute_gradient: bool = False):
        assert tuple(x.shape) == (self.N, 1), (tuple(x.shape), self.N)
        cost, grad = self._compute_cost_and_gradient(x, compute_gradient)
        cost = self.lam * cost
        if compute_gradient:
            return cost, self.lam * grad
        return cost


class RowTotalVariation(Prior):
    """Each row constant; cost = mean over adjacent rows of sqrt(diff^2 + eps^2)."""

    def __init__(self, nz: int = 70, nx: int = 70, epsilon: float = 0.1, device=None):
        super().__init__(nz, nx, device)
        self.epsilon = epsilon
        self.N = nz + 1
        self.lam = 1e-8

    def _prep(self):
        B = torch.zeros((self.nv, self.N), dtype=F64, device=self.device)
        for r in range(self.nz):
            B[r * self.nx:(r + 1) * self.nx, r] = 1.0
        B[-1, -1] = 1.0   # min_vel
        self.basis_vectors = B

    def _compute_cost_and_gradient(self, x, compute_gradient):
        nz = self.nz
        diff = torch.diff(x[:nz], dim=0)
        per = torch.sqrt(diff ** 2 + self.epsilon ** 2)
        cost = per.mean()
        grad = None
        if compute_gradient:
            sign = diff / per
            grad = torch.zeros_like(x)
            grad[0] = -sign[0]
            grad[1:nz - 1] = sign[:-1] - sign[1:]
            grad[nz - 1] = sign[-1]
            grad = grad / (nz - 1)
        return cost, grad


class TotalVariation(Prior):
    """2-D smoothed TV: mean of f(d) over vertical and horizontal neighbour differences,
    f(d) = sqrt(d^2 + eps^2) (``cost_func``/``grad_cost_func`` replaceable)."""

    def __init__(self, nz: int = 70, nx: int = 70, epsilon: float = 0.1, device=None):
        super().__init__(nz, nx, device)
        self.epsilon = epsilon
        self.N = self.nv
        self.lam = 1e-8
        self.cost_func = lambda d: torch.sqrt(d ** 2 + self.epsilon ** 2)
        self.grad_cost_func = lambda d: d / torch.sqrt(d ** 2 + self.epsilon ** 2)

    def _prep(self):
        self.basis_vectors = self._identity_basis()

    def batched_cost_and_gradient(self, X: torch.Tensor):
        """lambda * cost and its gradient for M unknown vectors (M, N) at once (the
        default sqrt(d^2 + eps^2) penalty).  CUDA tensors go through the library's fused
        kernel (seis_tv_prior: each model's result independent of M)."""
        M = X.shape[0]
        if X.is_cuda:
            import ctypes

            from ._lib import SeisError, load
            lib = load()
            Xc = X.contiguous()
            cost = torch.empty(M, dtype=F64, device=X.device)
            grad = torch.empty_like(Xc)
            st = torch.cuda.current_stream(X.device).cuda_stream
            rc = lib.seis_tv_prior(M, self.nz, self.nx, float(self.epsilon), float(self.lam),
                                   ctypes.c_void_p(Xc.data_ptr()), ctypes.c_void_p(cost.data_ptr()),
                                   ctypes.c_void_p(grad.data_ptr()), ctypes.c_void_p(st))
            if rc != 0:
                raise SeisError(rc, (lib.seis_last_error(None) or b"").decode())
            return cost, grad
        m = X[:, :-1].reshape(M, self.nz, self.nx)
        d1 = torch.diff(m, dim=1)
        d2 = torch.diff(m, dim=2)
        n = d1[0].numel() + d2[0].numel()
        e2 = self.epsilon ** 2
        s1 = torch.sqrt(d1 ** 2 + e2)
        s2 = torch.sqrt(d2 ** 2 + e2)
        cost = (s1.reshape(M, -1).sum(1) + s2.reshape(M, -1).sum(1)) / n
        g1 = d1 / s1 / n
        g2 = d2 / s2 / n
        gm = torch.zeros_like(m)
        gm[:, 1:, :] += g1
        gm[:, :-1, :] -= g1
        gm[:, :, 1:] += g2
        gm[:, :, :-1] -= g2
        grad = torch.cat((gm.reshape(M, -1), torch.zeros((M, 1), dtype=F64, device=X.device)), dim=1)
        return self.lam * cost, self.lam * grad

    def _compute_cost_and_gradient(self, x, compute_gradient):
        m = x[:-1].reshape(self.nz, self.nx)
        d1 = torch.diff(m, dim=0)
        d2 = torch.diff(m, dim=1)
        diff = torch.cat((d1.reshape(-1), d2.reshape(-1)))
        cost = self.cost_func(diff).mean()
        grad = None
        if compute_gradient:
            n = diff.numel()
            g1 = self.grad_cost_func(d1) / n
            g2 = self.grad_cost_func(d2) / n
            gm = torch.zeros_like(m)
            gm[1:, :] += g1
            gm[:-1, :] -= g1
            gm[:, 1:] += g2
            gm[:, :-1] -= g2
            grad = torch.cat((gm.reshape(-1), torch.zeros(1, dtype=F64, device=x.device))).reshape(x.shape)
        return cost, grad


class SquaredExponential(Prior):
    """Gaussian-process prior, cost x^T P x with P = K^-1 (squared-exponential kernel plus a
    constant, a depth slope and a nugget); ``transform`` switches to the scaled SVD modes of K."""

    def __init__(self, nz: int = 70, nx: int = 70, device=None, transform: bool = False, svd_cutoff: float = 0.0):
        super().__init__(nz, nx, device)
        self.length_scale = math.log(32.4)
        self.noise = 0.1
        self.sigma = 183.4
        self.sigma_mean = 520.0
        self.sigma_slope = 31.4
        self.transform = transform
        self.svd_cutoff = svd_cutoff
        self.P = None
        self.N = self.nv
        self.lam = 1e-8

    def covariance(self) -> torch.Tensor:
        nz, nx = self.nz, self.nx
        zc = torch.arange(nz, dtype=F64, device=self.device) - nz // 2
        xc = torch.arange(nx, dtype=F64, device=self.device) - nx // 2
        y = zc[:, None].expand(nz, nx).reshape(-1, 1)
        x = xc[None, :].expand(nz, nx).reshape(-1, 1)
        d2 = (x - x.T) ** 2 + (y - y.T) ** 2
        K = (self.sigma ** 2) * torch.exp(-d2 / (2 * self.length_scale ** 2))
        K = K + self.sigma_mean ** 2
        K = K + (self.sigma_slope ** 2) * (y @ y.T)
        K = K + (self.noise ** 2) * torch.eye(nz * nx, dtype=F64, device=self.device)
        return K

    def _prep(self):
        K = self.covariance()
        self.P = torch.linalg.inv(K)
        if self.transform:
            U, s, _ = torch.linalg.svd(K)
            keep = s > self.svd_cutoff
            B = U[:, keep] * torch.sqrt(s[keep])[None, :]
            B = torch.nn.functional.pad(B, (0, 1, 0, 1))
            B[-1, -1] = 1.0
            self.P = torch.eye(B.shape[1] - 1, dtype=F64, device=self.device)
            self.basis_vectors = B
        else:
            self.basis_vectors = self._identity_basis()
        self.N = self.basis_vectors.shape[1]

    def _compute_cost_and_gradient(self, x, compute_gradient):
        xv = x[:-1, :]
        Px = self.P @ xv
        cost = (xv.T @ Px)[0, 0]
        grad = None
        if compute_gradient:
            grad = 2 * torch.cat((Px, torch.zeros((1, 1), dtype=F64, device=x.device)))
        return cost, grad


def label_thresholded_components(a: np.ndarray, threshold: float, connectivity: int = 4):
    """Connected components of a grid where neighbours differ by <= threshold
    (core/seis_numerics.py:81-124; host SciPy, as in the reference)."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    h, w = a.shape
    idx = np.arange(h * w).reshape(h, w)
    offs = [(1, 0), (0, 1)] if connectivity == 4 else [(1, 0), (0, 1), (1, 1), (1, -1)]
    rows, cols = [], []
    for di, dj in offs:
        i0, i1 = max(0, -di), h - max(0, di)
        j0, j1 = max(0, -dj), w - max(0, dj)
        A = a[i0:i1, j0:j1]
        Bn = a[i0 + di:i1 + di, j0 + dj:j1 + dj]
        ok = np.abs(Bn - A) <= threshold
        rows.append(idx[i0:i1, j0:j1][ok])
        cols.append(idx[i0 + di:i1 + di, j0 + dj:j1 + dj][ok])
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    adj = coo_matrix((np.ones(len(r), dtype=bool), (r, c)), shape=(h * w, h * w)).tocsr()
    n, labels = connected_components(adj, directed=False, return_labels=True)
    return labels.reshape(h, w), n


class RestrictFlatAreas(Prior):
    """Areas that are flat (neighbour differences <= diff_threshold) in the starting
    model stay exactly flat: one basis vector per flat component (scaled to unit
    column sum), on top of an identity-basis underlying prior."""

    def __init__(self, underlying_prior: Prior, diff_threshold: float = 1.0):
        super().__init__(underlying_prior.nz, underlying_prior.nx, underlying_prior.device)
        self.underlying_prior = underlying_prior
        self.diff_threshold = diff_threshold
        self.N = self.nv
        self.lam = 1.0

    def _prep(self):
        self.underlying_prior.prep()
        self.basis_vectors = self.underlying_prior.basis_vectors
        self.N = self.nv

    def _adapt(self, velocity_guess):
        m = np.asarray(velocity_guess, dtype=np.float64).reshape(self.nz, self.nx)
        labels, count = label_thresholded_components(m, self.diff_threshold, connectivity=4)
        labels = labels.ravel()
        B = np.zeros((self.nz * self.nx, count), dtype=np.float64)
        B[np.arange(self.nz * self.nx), labels] = 1.0
        B = B[:, B.sum(axis=0) > 0]
        full = np.zeros((self.nv, B.shape[1] + 1))
        full[:-1, :-1] = B
        full[-1, -1] = 1.0
        full = full / full.sum(axis=0, keepdims=True)
        self.basis_vectors = torch.as_tensor(full, dtype=F64, device=self.device)
        self.N = self.basis_vectors.shape[1]

    def _compute_cost_and_gradient(self, x, compute_gradient):
        ux = self.basis_vectors @ x
        if compute_gradient:
            c, ug = self.underlying_prior.compute_cost_and_gradient(ux, True)
            return c, self.basis_vectors.T @ ug
        return self.underlying_prior.compute_cost_and_gradient(ux, False), None
