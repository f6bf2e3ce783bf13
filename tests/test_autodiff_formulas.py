"""Closed forms of the field-map gradients, pinned against torch autograd of a
dense complex128 model on the CPU (no GPU, no package code).

For ``y = E(f) (s_c x)`` with ``E_mn = A_mn exp(f_n t_m)`` the gradient of a
real loss with respect to the complex field map is ``conj(x) * E^H(t dy)``
summed over coils; for ``x = sum_c conj(s_c) E(f)^H y_c`` it is
``conj(dx) * E^H(t y)``.  The forward formula of mri-nufft's autodiff
(``autodiff.py:44-56``) multiplies by ``x`` instead of ``conj(x)``; the test
records that this differs from the derivative, which is what the CUDA path
implements.
"""

import torch


def _setup(seed=0, M=50, N=30, C=2):
    g = torch.Generator().manual_seed(seed)

    def c(*shape):
        return torch.complex(torch.randn(*shape, generator=g, dtype=torch.float64),
                             torch.randn(*shape, generator=g, dtype=torch.float64))

    t = torch.rand(M, generator=g, dtype=torch.float64)
    return c(M, N), t, 0.3 * c(N), c(C, N), c(N), c(C, M)


def _E(A, t, f):
    return A * torch.exp(t[:, None] * f[None, :])


def _rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def test_forward_field_map_gradient():
    A, t, f0, s, x, y0 = _setup()
    f = f0.clone().requires_grad_(True)
    y = torch.stack([_E(A, t, f) @ (s[c] * x) for c in range(s.shape[0])])
    torch.sum(torch.abs(y - y0) ** 2).backward()
    dy = 2 * (y.detach() - y0)
    Eh = _E(A, t, f0).conj().T
    back = sum(s[c].conj() * (Eh @ (t * dy[c])) for c in range(s.shape[0]))
    assert _rel(x.conj() * back, f.grad) < 1e-12
    assert _rel(x * back, f.grad) > 1e-1


def test_adjoint_field_map_gradient():
    A, t, f0, s, x0, y = _setup(1)
    f = f0.clone().requires_grad_(True)
    xa = sum(s[c].conj() * (_E(A, t, f).conj().T @ y[c]) for c in range(s.shape[0]))
    torch.sum(torch.abs(xa - x0) ** 2).backward()
    dx = 2 * (xa.detach() - x0)
    Eh = _E(A, t, f0).conj().T
    closed = dx.conj() * sum(s[c].conj() * (Eh @ (t * y[c])) for c in range(s.shape[0]))
    assert _rel(closed, f.grad) < 1e-12
