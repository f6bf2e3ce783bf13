"""Host-side kernel and grid parameters, identical to the rules the C library
applies in ``gbn_plan_create`` (``csrc/gbn_capi.cu``).

The exponential-of-semicircle parameters follow the published finufft rules
(Barnett, Magland & af Klinteberg, SISC 2019): at upsampling factor 2,
``w = ceil(-log10(eps / 10))`` and ``beta = c(w) w`` with c = 2.20, 2.26,
2.38 for w = 2, 3, 4 and 2.30 above; for another factor sigma,
``w = ceil(-ln(eps) / (pi sqrt(1 - 1/sigma)))`` and
``beta = 0.97 pi w (1 - 1/(2 sigma))``; w is clamped to [2, 16].  The fine
grid is the smallest even 2-3-5-smooth size >= max(ceil(sigma N), 2 w).
"""

from __future__ import annotations

import math


def kernel_params(eps: float, sigma: float = 2.0):
    if sigma == 2.0:
        w = math.ceil(-math.log10(eps / 10.0))
    else:
        w = math.ceil(-math.log(eps) / (math.pi * math.sqrt(1.0 - 1.0 / sigma)))
    w = max(2, min(16, w))
    if sigma == 2.0:
        c = {2: 2.20, 3: 2.26, 4: 2.38}.get(w, 2.30)
        beta = c * w
    else:
        beta = 0.97 * math.pi * w * (1.0 - 1.0 / (2.0 * sigma))
    return w, beta


def next_smooth_even(n: int) -> int:
    if n <= 2:
        return 2
    if n % 2:
        n += 1
    while True:
        r = n
        for p in (2, 3, 5):
            while r % p == 0:
                r //= p
        if r == 1:
            return n
        n += 2


def fine_shape(shape, eps=1e-6, sigma=2.0, spread_only=False):
    w, _ = kernel_params(eps, sigma if sigma > 1 else 2.0)
    if spread_only:
        return tuple(int(n) for n in shape)
    return tuple(next_smooth_even(max(math.ceil(sigma * n), 2 * w)) for n in shape)


def fine_cells(shape, eps=1e-6, sigma=2.0, spread_only=False) -> int:
    g = 1
    for n in fine_shape(shape, eps, sigma, spread_only):
        g *= n
    return g
