"""The allocation-free per-pair entry point (motex_gpu_extract_pair_static).

It exists for callers that cannot call cudaMalloc (code inside another
framework's memory pool, code with a fixed memory budget, plug-ins handed
only device buffers): its scratch is a static device array.  Here it is
called through the C ABI with device buffers the test owns and must give
the same u / v as the allocating entry point motex_gpu_extract_pair, on two
calls in a row (the second call of a different size, so stale scratch from
the first would show).  Collected last on purpose.
"""
import ctypes as C
import random

import pytest


def _static_call(native, d, l, e, alphabet, p, t, u0=None, v0=None):
    import torch
    lib = native.load_library()
    dev = torch.device("cuda:0")
    dp = torch.tensor(list(p.encode()), dtype=torch.uint8, device=dev)
    dt = torch.tensor(list(t.encode()), dtype=torch.uint8, device=dev)
    du = torch.tensor(u0 or [0] * len(p), dtype=torch.int32, device=dev)
    dv = torch.tensor(v0 or [0] * len(p), dtype=torch.int32, device=dev)
    prm = native.make_params(d, l, e)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = lib.motex_gpu_extract_pair_static(C.byref(prm), alphabet.encode(), dp.data_ptr(), len(p), dt.data_ptr(),
                                           len(t), du.data_ptr(), dv.data_ptr(), C.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, du.cpu().tolist(), dv.cpu().tolist()


def _case(rng, alphabet, l, e, m, n):
    p = "".join(rng.choice(alphabet) for _ in range(m))
    t = "".join(rng.choice(alphabet) for _ in range(n))
    for _ in range(4):                                 # near-copies of factors of p in t
        a, b = rng.randint(0, m - l), rng.randint(0, n - l)
        w = list(p[a:a + l])
        for _ in range(rng.randint(0, e)):
            w[rng.randrange(l)] = rng.choice(alphabet)
        t = t[:b] + "".join(w) + t[b + l:]
    return p, t


@pytest.mark.gpu
def test_static_matches_allocating_entry_point_twice(native_built):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    ctx = native_built.Context(0)
    try:
        rng = random.Random(2024)
        calls = [(1, 15, 3, "ACGTN", 3000, 20000), (0, 12, 2, "ARNDCQEGHILKMFPSTWYVOUBZJX*", 700, 5000)]
        for d, l, e, alphabet, m, n in calls:
            p, t = _case(rng, alphabet, l, e, m, n)
            rc, u, v = _static_call(native_built, d, l, e, alphabet, p, t)
            assert rc == 0
            ur, vr = ctx.extract_pair(p, t, native_built.make_params(d, l, e))
            assert u == ur and v == vr
            assert sum(v) > 0
    finally:
        ctx.close()


@pytest.mark.gpu
def test_static_rejects_oversize_and_bad_symbols(native_built):
    pytest.importorskip("torch")
    rc, _, _ = _static_call(native_built, 0, 8, 1, "ACGT", "A" * 40000, "ACGT" * 10)
    assert rc == -4                                     # m above the 32768 limit
    rc, u, v = _static_call(native_built, 0, 4, 1, "ACGT", "ACGTACGTQQ", "ACGTACGT")
    assert rc == -1 and sum(u) == 0 and sum(v) == 0      # Q is not in the alphabet
