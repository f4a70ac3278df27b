"""Host logic of the serving and batch entry points (no GPU needed).

Requests that can never fit the budget are rejected before any device work;
runs that fail (here: no CUDA device) surface their status through the
request and batch objects; the device-memory estimate grows with the field.
"""
import pytest

from ccf_gb300 import CCF, CCFError, Server, _lib
from ccf_gb300.ccf import _bare

SMALL = dict(kappa_tot=0.3, kappa_star=0.3, shear=0.1, num_stars=100, num_phi=100, num_branches=1, random_seed=1)


def test_estimate_grows_with_the_field():
    base = _bare(**SMALL).estimate_device_bytes()
    more_stars = _bare(**{**SMALL, "num_stars": 1000}).estimate_device_bytes()
    more_phi = _bare(**{**SMALL, "num_phi": 1000}).estimate_device_bytes()
    assert 0 < base < more_stars
    assert base < more_phi
    # outputs dominate a long run: at least its root and 1/mu arrays
    d = _bare(**{**SMALL, "num_phi": 1000}).estimate_device_bytes()
    assert d >= 200 * 1001 * 24


def test_estimate_rejects_invalid_parameters():
    with pytest.raises(CCFError):
        _bare(**{**SMALL, "num_phi": 101}).estimate_device_bytes()


def test_server_rejects_a_request_larger_than_the_budget():
    s = Server(slots=2, hbm_budget=1 << 20)   # 1 MiB: nothing fits
    try:
        rid = s.submit(**SMALL)
        assert s.wait(rid, timeout=30) == _lib.STATUS_CODES["CCF_ERR_BUDGET"]
        info = s.info(rid)
        assert info["state"] == _lib.REQUEST_REJECTED
        st = s.stats()
        assert st["rejected"] == 1 and st["admitted"] == 0 and st["bytes_in_use"] == 0
        with pytest.raises(CCFError):
            s.field(rid)
        s.release(rid)
        assert s.stats()["submitted"] == 1
    finally:
        s.close()


def test_server_refuses_invalid_submissions_and_configs():
    s = Server(slots=1, hbm_budget=1 << 30)
    try:
        with pytest.raises(CCFError):
            s.submit(**{**SMALL, "num_branches": 3})   # num_phi not a multiple of 2 * num_branches
        assert s.stats()["submitted"] == 0
        with pytest.raises(CCFError):
            s.info(12345)
    finally:
        s.close()
    for slots, budget in ((0, 1 << 30), (1, 0)):
        with pytest.raises(CCFError):
            Server(slots=slots, hbm_budget=budget)


def test_server_reports_a_failed_run():
    """Without a GPU the admitted request runs and fails; the server keeps
    its handle with the error and returns its bytes to the budget on release."""
    if _has_gpu():
        pytest.skip("this checks the failure path, which needs a host without a GPU")
    s = Server(slots=1, hbm_budget=1 << 34)
    try:
        rid = s.submit(**SMALL)
        status = s.wait(rid, timeout=60)
        assert status == _lib.STATUS_CODES["CCF_ERR_NO_DEVICE"]
        info = s.info(rid)
        assert info["state"] == _lib.REQUEST_FAILED
        assert info["t_submit"] <= info["t_start"] <= info["t_end"]
        f = s.field(rid)
        assert "No CUDA capable devices" in f.last_error()
        assert s.stats()["bytes_in_use"] == info["bytes"]
        s.release(rid)
        st = s.stats()
        assert st["bytes_in_use"] == 0 and st["failed"] == 1
    finally:
        s.close()


def test_async_batch_reports_the_run_status():
    if _has_gpu():
        pytest.skip("this checks the failure path, which needs a host without a GPU")
    from ccf_gb300 import submit_batch
    fields = [CCF(**SMALL), CCF(**{**SMALL, "random_seed": 2})]
    job = submit_batch(fields)
    assert job.wait() is False
    assert job.done()
    assert all(f.last_status == _lib.STATUS_CODES["CCF_ERR_NO_DEVICE"] for f in fields)


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
