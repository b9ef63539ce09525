"""Failure detection on the GPU without a GPU fault: every pipeline wait in
the library's kernels is a bounded mbarrier wait that, when it runs out,
records an error code in a device word and lets the kernel return.  The
self-test runs that same wait with a 100 ms limit on a barrier nothing
arrives on; the host must read the timeout, every waiting thread must have
returned, and the context must stay usable."""
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import ugemm_gb300 as ug  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ug.build()
    ug.load()


def test_bounded_wait_runs_out_and_the_context_stays_usable():
    status, code, threads, seconds = ug.selftest_wait_timeout()
    assert status == ug.ERR_TIMEOUT
    assert code == 1                 # a pipeline stage never filled
    assert threads == 64             # every waiter gave up and returned
    assert 0.09 <= seconds < 5.0     # after the limit, not never
    # the context still runs GEMMs, in both forms, correctly
    g = torch.Generator(device="cuda").manual_seed(4)
    A = torch.rand((300, 200), device="cuda", generator=g)
    B = torch.rand((200, 260), device="cuda", generator=g)
    ref = A.double() @ B.double()
    for prec in ("simt", "bf16x6"):
        C = ug.gemm(A, B, precision=prec)
        torch.cuda.synchronize()
        assert float(torch.linalg.norm(C.double() - ref) / torch.linalg.norm(ref)) < 2e-6
    # and a second run reports the same again (the self-test's error word is its own)
    assert ug.selftest_wait_timeout()[:3] == (ug.ERR_TIMEOUT, 1, 64)
