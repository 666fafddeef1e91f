"""rpg_session_sieve_noalloc: sieving without allocating device memory.

Some callers cannot allocate when they sieve: engines that reserve all of
their device memory up front and hand it out from their own pool, and
latency-bound loops that cannot afford cudaMalloc/cudaFree (which may
synchronize the device).  They create a session ahead of time and then call
this entry point with their own device arrays.  Here it is called through the
C ABI twice in a row, into caller-owned arrays, and each result must equal
what rpg_sieve_run delivers for the same curve, bound and denominators (the
survivor sets are integer data, so equality is exact).  A timed-out device
wait is reported through the caller's count (UINT64_MAX); the test makes that
timeout on the host, through the library's injection hook, not on the GPU.
"""

import ctypes

import pytest

pytestmark = pytest.mark.gpu

RECORD = "247747600 -985905640 567207969 2396040466 52485681 -470135160 82342800".split()


def _entry(rpg):
    fn = rpg.load().rpg_session_sieve_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    return fn


def _dense_coefficients():
    # 1 + P x with P the product of the 32 largest primes below 512: every
    # site survives the reference plan.
    primes = [p for p in range(2, 512) if all(p % q for q in range(2, int(p ** 0.5) + 1))]
    product = 1
    for p in primes[-32:]:
        product *= p
    return ["1", str(product)]


CASES = [("fast", RECORD, 100_000, 1, 3000), ("reference", RECORD, 100_000, 1, 3000),
         ("reference", "dense", 5000, 1, 2), ("fast", ["1", "3", "0", "-7", "2"], 4097, 1, 70000)]


@pytest.mark.parametrize("plan,coeffs,bound,first,last", CASES,
                         ids=["fast-record", "reference-record", "reference-dense", "fast-batches"])
def test_noalloc_matches_sieve_run(rpg, plan, coeffs, bound, first, last):
    torch = pytest.importorskip("torch")
    if coeffs == "dense":
        coeffs = _dense_coefficients()
    a_ref, d_ref, _ = rpg.sieve(coeffs, bound, first, last, plan=plan)
    expected = sorted(zip(a_ref.tolist(), d_ref.tolist()))
    entry = _entry(rpg)
    session = rpg.Session(coeffs, bound, plan=plan)
    capacity = 2 * len(expected) + 1024
    a = torch.empty(capacity, dtype=torch.int64, device="cuda")
    d = torch.empty(capacity, dtype=torch.int32, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    try:
        for _ in range(2):  # two calls in a row share the scratch array
            a.fill_(-1)
            d.fill_(-1)
            torch.cuda.synchronize()
            status = entry(session._handle, first, last, a.data_ptr(), d.data_ptr(), capacity,
                           count.data_ptr(), None)
            assert status == 0, rpg.load().rpg_last_error().decode()
            torch.cuda.synchronize()
            n = int(count.item())
            assert n == len(expected) and n <= capacity
            got = sorted(zip(a[:n].cpu().tolist(), d[:n].cpu().tolist()))
            assert got == expected
    finally:
        session.close()


def test_noalloc_rejects_more_than_its_scratch_covers(rpg):
    torch = pytest.importorskip("torch")
    entry = _entry(rpg)
    session = rpg.Session(["1", "0", "1"], 10, plan="fast")
    buf = torch.empty(64, dtype=torch.int64, device="cuda")
    try:
        status = entry(session._handle, 1, 16_777_217, buf.data_ptr(), buf.data_ptr(), 8,
                       buf.data_ptr(), None)
        assert status == 1
        assert "at most 16777216" in rpg.load().rpg_last_error().decode()
    finally:
        session.close()


def test_noalloc_reports_a_timeout_through_the_count(rpg, monkeypatch):
    torch = pytest.importorskip("torch")
    coeffs, bound, first, last = RECORD, 100_000, 1, 3000
    a_ref, d_ref, _ = rpg.sieve(coeffs, bound, first, last, plan="fast")
    expected = sorted(zip(a_ref.tolist(), d_ref.tolist()))
    entry = _entry(rpg)
    session = rpg.Session(coeffs, bound, plan="fast")
    capacity = 2 * len(expected) + 1024
    a = torch.empty(capacity, dtype=torch.int64, device="cuda")
    d = torch.empty(capacity, dtype=torch.int32, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    try:
        # a launch whose bounded wait gave up: the count becomes the sentinel
        monkeypatch.setenv("RPG_TEST_INJECT_NOALLOC_TIMEOUT", "1")
        status = entry(session._handle, first, last, a.data_ptr(), d.data_ptr(), capacity,
                       count.data_ptr(), None)
        assert status == 0, rpg.load().rpg_last_error().decode()
        torch.cuda.synchronize()
        assert int(count.item()) == -1  # UINT64_MAX read as int64
        # the next call clears the shared error word and is complete again
        monkeypatch.delenv("RPG_TEST_INJECT_NOALLOC_TIMEOUT")
        status = entry(session._handle, first, last, a.data_ptr(), d.data_ptr(), capacity,
                       count.data_ptr(), None)
        assert status == 0, rpg.load().rpg_last_error().decode()
        torch.cuda.synchronize()
        n = int(count.item())
        assert n == len(expected)
        assert sorted(zip(a[:n].cpu().tolist(), d[:n].cpu().tolist())) == expected
    finally:
        session.close()


@pytest.mark.parametrize("plan,bound", [("fast", 10**11), ("reference", 10**11)])
def test_noalloc_rejects_rows_wider_than_one_launch(rpg, plan, bound):
    torch = pytest.importorskip("torch")
    entry = _entry(rpg)
    session = rpg.Session(["1", "3", "0", "-7", "2"], bound, plan=plan)
    buf = torch.empty(64, dtype=torch.int64, device="cuda")
    try:
        status = entry(session._handle, 1, 4, buf.data_ptr(), buf.data_ptr(), 8, buf.data_ptr(),
                       None)
        assert status == 1
        assert "numerator bound is too large" in rpg.load().rpg_last_error().decode()
    finally:
        session.close()
