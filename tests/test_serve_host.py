"""Server request validation on the host (no GPU work happens at submit)."""
import pytest

from dgcuda_gb300 import _ffi
from dgcuda_gb300.serve import Server, request


@pytest.fixture
def server(native):
    s = Server(budget_bytes=64 << 20, max_active=8)
    yield s
    s.close()


@pytest.mark.parametrize("bad,status", [
    (dict(order=7), _ffi.ERR_UNSUPPORTED),
    (dict(t_end=0.0), _ffi.ERR_INVALID),
    (dict(n=0), _ffi.ERR_INVALID),
    (dict(precision=_ffi.FP32_BF16X3), _ffi.ERR_UNSUPPORTED),
    (dict(cfl=0.0), _ffi.ERR_INVALID),
])
def test_invalid_requests_rejected(bad, status, server):
    kw = dict(n=8, order=2, equation=_ffi.EULER, ic=_ffi.IC_VORTEX, t_end=0.1)
    kw.update(bad)
    with pytest.raises(_ffi.DgxError) as ei:
        server.submit(request(**kw))
    assert ei.value.status == status


def test_request_larger_than_budget_rejected(server):
    with pytest.raises(_ffi.DgxError) as ei:
        server.submit(request(n=2048, order=4, equation=_ffi.EULER, ic=_ffi.IC_VORTEX))
    assert ei.value.status == _ffi.ERR_BUSY
    st = server.stats()
    assert st["submitted"] == 0 and st["queued"] == 0
