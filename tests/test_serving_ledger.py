"""Admission of the served form against its HBM budget, on the host.

The server's GPU work is replaced by stand-ins (a sorted trajectory that
only carries its byte charge, a solve that finishes after a few units), so
that the admission, pre-building, pooling and eviction logic runs on the
CPU: pre-built trajectories plus admitted requests never exceed the budget,
a request that would overflow waits for a slot to free up, idle pooled
trajectories are freed to admit a request of another protocol, and a
request larger than the whole budget is refused.
"""

import types

import numpy as np
import pytest


@pytest.fixture()
def serving(pkg, monkeypatch):
    from mrinufft_gb300 import serving as sv

    class FakeSolve:
        def __init__(self, server, req, pset, stream, nbytes):
            self.req, self.pset, self.bytes = req, pset, int(nbytes)
            self.units = 3
            self.image, self.L = "image", "L"
            self.event = types.SimpleNamespace(query=lambda: True)

        def step(self):
            self.units -= 1
            return self.units > 0

    def fake_build(self, req, stream):
        p = types.SimpleNamespace(bytes=self._pset_bytes(req))
        self.ledger.add_resident(p.bytes)
        self.built.append(p)
        return p

    monkeypatch.setattr(sv, "_Solve", FakeSolve)
    monkeypatch.setattr(sv.ReconServer, "_build_plan", fake_build)
    monkeypatch.setattr(sv.ReconServer, "_stream", lambda self, i: None)
    monkeypatch.setattr(sv.torch.cuda, "synchronize", lambda *a, **k: None)
    monkeypatch.setattr(sv._lib, "load", lambda: None)
    return sv


def _req(sv, rid, shape=(64, 64), M=4000, C=8, key="a", smaps_key=None):
    return sv.ReconRequest(rid=rid, samples=np.zeros((M, len(shape)), np.float32), shape=shape,
                           kspace=np.zeros((C, M), np.complex64),
                           smaps=np.zeros((C, *shape), np.complex64), traj_key=key,
                           smaps_key=smaps_key, seed=rid)


def _server(sv, budget, **kw):
    srv = sv.ReconServer(hbm_budget_bytes=budget, device=0, **kw)
    srv.built = []
    return srv


def _drive(srv, reqs):
    for r in reqs:
        srv.submit(r)
    for r in reqs:
        r._x0.result()
    peak_active = 0
    while not srv.idle():
        srv.tick()
        peak_active = max(peak_active, len(srv.active) + len(srv.finishing))
        assert srv.ledger.total <= srv.budget
    return peak_active


def test_prewarmed_plus_admitted_never_exceed_budget(serving):
    sv = serving
    reqs = [_req(sv, i, key="ab"[i % 2]) for i in range(12)]
    pset = sv.plan_set_bytes((64, 64), 4000, 8)
    solve = sv.solve_bytes((64, 64), 4000, 8)
    budget = 3 * pset + 2 * solve
    srv = _server(sv, budget, max_active=8)
    srv.prewarm(reqs)
    assert srv.ledger.total <= budget
    assert len(srv.built) == 3  # building stops at the budget
    peak = _drive(srv, reqs)
    assert len(srv.done) == len(reqs)
    assert srv.ledger.peak <= budget
    assert peak <= 3
    assert srv.ledger.active == 0


def test_other_protocol_evicts_idle_pooled_plans(serving):
    sv = serving
    pset = sv.plan_set_bytes((64, 64), 4000, 8)
    solve = sv.solve_bytes((64, 64), 4000, 8)
    srv = _server(sv, 2 * pset + solve, max_active=4)
    srv.prewarm([_req(sv, 0, key="a")], per_key=2)
    assert len(srv.plans[srv._key(_req(sv, 0, key="a"))]) == 2
    _drive(srv, [_req(sv, 1, key="b")])
    assert len(srv.done) == 1
    assert srv.ledger.peak <= srv.budget


def test_resident_coil_maps_are_charged_once(serving):
    sv = serving
    pset = sv.plan_set_bytes((64, 64), 4000, 8)
    srv = _server(sv, 10 * pset, max_active=4)
    _drive(srv, [_req(sv, i, smaps_key="maps") for i in range(5)])
    assert srv.ledger.resident == pset * len(srv.built) + sv.smaps_bytes((64, 64), 8)


def test_request_larger_than_budget_is_refused(serving):
    sv = serving
    srv = _server(sv, sv.plan_set_bytes((64, 64), 4000, 8) // 2, max_active=4)
    with pytest.raises(RuntimeError, match="HBM budget"):
        _drive(srv, [_req(sv, 0)])
