"""CPU oracle of the GB300 NUFFT backend — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` (plus ``bench.py --impl reference``) may import this package.
It is the checker, never part of the product path:

* ``ndft``      exact FP64 NDFT (restates ``nudft_numpy.py``), pinned to
                golden vectors produced by the reference itself;
* ``operator``  operator-level semantics (SENSE, batches, density, DC, CG,
                power method) of ``operators/base.py`` / ``extras/optim.py``
                on the NDFT;
* ``esnufft``   a C / OpenMP exponential-of-semicircle NUFFT (the published
                finufft algorithm the reference delegates to), used for the
                pipe density check and as the timed CPU baseline.
"""
