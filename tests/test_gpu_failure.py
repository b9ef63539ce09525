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


@pytest.mark.parametrize("prec", ["bf16x6", "fp16x3", "simt"])
def test_stale_timeout_is_reported_once_and_does_not_stop_later_calls(prec):
    """A timeout left in the device-pointer calls' error word -- planted with a
    host copy, as a kernel wait that ran out would leave it; nothing faults
    or hangs -- must neither make the next call's kernels give up (C must
    still be right) nor be lost: ugemm_check reports it exactly once."""
    ug.check()  # start clean
    g = torch.Generator(device="cuda").manual_seed(12)
    M, N, K = 1100, 900, 1500   # deep enough for chunk drains, more tiles than one wave
    A = torch.rand((M, K), device="cuda", generator=g) * 2 - 1
    B = torch.rand((K, N), device="cuda", generator=g) * 2 - 1
    ref = ug.ref64("N", "N", A, B)
    assert ug.load().ugemm_debug_set_error_word(0, 3) == ug.OK
    C = torch.full((M, N), float("nan"), device="cuda")
    ug.sgemm_dev("N", "N", M, N, K, 1.0, A, K, B, N, 0.0, C, N, precision=prec)
    torch.cuda.synchronize()
    assert float(torch.linalg.norm(C.double() - ref) / torch.linalg.norm(ref)) < 2e-6
    with pytest.raises(ug.UgemmError) as err:
        ug.check()
    assert err.value.status == ug.ERR_TIMEOUT
    assert "code 3" in str(err.value)
    ug.check()  # reported once: the word is clean again
    # the backward path folds the word the same way
    assert ug.load().ugemm_debug_set_error_word(0, 2) == ug.OK
    dA = torch.zeros((M, K), device="cuda")
    ug.sgemm_backward("N", "N", M, N, K, 1.0, A, K, B, N, C, N, 0.0, dA, K, 0.0, None, N,
                      precision=prec)
    torch.cuda.synchronize()
    refA = ug.ref64("N", "T", C, B)
    assert float(torch.linalg.norm(dA.double() - refA) / torch.linalg.norm(refA)) < 2e-6
    with pytest.raises(ug.UgemmError):
        ug.check()
    ug.check()
