"""Serving and asynchronous batches on the GPU.

Each request of the server runs on its own handle, engine and stream; the
solver is deterministic (Jacobi sweeps, fixed cluster shapes), so a field's
results are the same bits whether it runs alone or while other requests run
beside it.  The memory budget bounds how many requests are admitted at once.
"""
import numpy as np
import pytest

from ccf_gb300 import CCF, Server, run_batch, submit_batch, _lib

pytestmark = pytest.mark.gpu

FIELDS = [
    dict(kappa_tot=0.3, kappa_star=0.3, shear=0.1, num_stars=60, num_phi=64, num_branches=2, random_seed=11),
    dict(kappa_tot=0.45, kappa_star=0.35, shear=0.35, mass_function="salpeter", m_lower=0.08, m_upper=1.5,
         m_solar=4.954984, rectangular=1, num_stars=120, num_phi=64, num_branches=4, random_seed=12),
    dict(kappa_tot=0.5, kappa_star=0.4, shear=0.25, mass_function="kroupa", m_lower=0.08, m_upper=1.5,
         rectangular=1, num_stars=200, num_phi=96, num_branches=4, random_seed=13),
    dict(kappa_tot=0.2, kappa_star=0.15, shear=0.5, mass_function="uniform", m_lower=0.1, m_upper=2, num_stars=90,
         num_phi=48, num_branches=3, random_seed=14),
]


def _collect(server, rid):
    assert server.wait(rid) == 0, server.field(rid).last_error()
    r = server.field(rid).results(stars=False)
    out = {k: r[k].copy() for k in ("ccs", "caustics", "errs")}
    server.release(rid)
    return out


def test_results_alone_equal_results_in_the_mix():
    alone = []
    s = Server(slots=1, hbm_budget=8e9)
    try:
        for f in FIELDS:
            alone.append(_collect(s, s.submit(**f)))
    finally:
        s.close()
    mix = Server(slots=4, hbm_budget=8e9)
    try:
        ids = [mix.submit(**f) for f in FIELDS]
        infos = []
        together = []
        for rid in ids:
            assert mix.wait(rid) == 0
            infos.append(mix.info(rid))
            together.append(_collect(mix, rid))
        # the requests did overlap on the device
        starts = [i["t_start"] for i in infos]
        ends = [i["t_end"] for i in infos]
        assert max(starts) < min(ends)
    finally:
        mix.close()
    for a, b, f in zip(alone, together, FIELDS):
        for k in ("ccs", "caustics", "errs"):
            assert np.array_equal(a[k], b[k]), (f, k)
    # and the same as a plain CCF run of that field
    c = CCF(**FIELDS[2])
    assert c.run(-1), c.last_error()
    r = c.results(stars=False)
    assert np.array_equal(r["ccs"], alone[2]["ccs"])


def test_budget_bounds_the_admitted_requests():
    fields = [dict(FIELDS[1], random_seed=100 + i) for i in range(5)]
    est = max(CCF(**f).estimate_device_bytes() for f in fields)
    s = Server(slots=4, hbm_budget=int(2.5 * est))   # room for two at a time
    try:
        ids = [s.submit(**f) for f in fields]
        infos = []
        for rid in ids:
            assert s.wait(rid) == 0
            infos.append(s.info(rid))
            assert s.stats()["bytes_in_use"] <= 2.5 * est
            s.release(rid)
        st = s.stats()
        assert st["completed"] == 5 and st["bytes_in_use"] == 0
        # never more than two running at once
        for i in infos:
            t = i["t_start"]
            concurrent = sum(1 for j in infos if j["t_start"] <= t < j["t_end"])
            assert concurrent <= 2
        assert st["deferred"] >= 1
    finally:
        s.close()


def test_submitted_batch_equals_run_batch():
    a = [CCF(**f) for f in FIELDS]
    assert run_batch(a)
    b = [CCF(**f) for f in FIELDS]
    job = submit_batch(b)
    assert job.wait()
    for x, y in zip(a, b):
        rx, ry = x.results(stars=False), y.results(stars=False)
        assert np.array_equal(rx["ccs"], ry["ccs"])
        assert np.array_equal(rx["caustics"], ry["caustics"])
