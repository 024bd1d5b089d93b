"""The allocation-free walker statistics entry point.

Callers that cannot allocate device memory (a host program whose own pool
owns all GPU memory) use tdvmc_reduce_walkers_noalloc with device arrays
they already own; its partial sums live in a fixed static device array.
This test drives it through the C ABI and checks it against
tdvmc_reduce_stats on the same walkers, at the FP64 tolerance of the other
parity tests (1e-12 relative), on two calls in a row, and checks that the
calls take no device memory (free device memory unchanged across them).
Cases: many walkers, fewer walkers than partial-sum blocks (one walker per
block), and p = 32, where the second pass fills the static array exactly.
The file name sorts last so a stop-at-first-failure run has run every other
test first.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


@pytest.mark.parametrize("nw,p", [(3001, 30), (5, 30), (700, 32)])
def test_noalloc_statistics_match_reduce_stats(nw, p):
    torch = pytest.importorskip("torch")
    import tdvmc_gb300 as T
    from tdvmc_gb300 import _native as N
    lib = N.load()
    dim, n, L = 3, 64, 6.0
    rng = np.random.default_rng(3 + nw)
    s = T.BosonsBulk(dim, n, p, L, nw, system_params=(1.0, 1.0), potential="lj", hbar2_2m=0.09, precision="fp64")
    r = np.linspace(0, L / 2, p)
    uR = -0.5 * (1.1 / np.maximum(r, 0.5)) ** 5
    uR -= uR[-1]
    s.SetParameters(uR, 0.02 * rng.normal(size=p))
    s.SetWalkers(rng.uniform(-L / 2, L / 2, size=(nw, dim, n)))
    f = s.CalculateExpectationValues()
    ref = s.ReduceStatistics()

    dev = torch.device("cuda")
    O = torch.tensor(f["O"], dtype=torch.float64, device=dev).contiguous()
    E = torch.tensor(f["eloc"], dtype=torch.float64, device=dev).contiguous()
    outs = [torch.empty(k, dtype=torch.float64, device=dev) for k in (p, 2, p * p, p, p)]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call():
        return lib.tdvmc_reduce_walkers_noalloc(C.c_void_p(O.data_ptr()), C.c_void_p(E.data_ptr()), nw, p,
                                                *[C.c_void_p(t.data_ptr()) for t in outs], stream)

    # warm-up of everything the checks below run: the first call on a device looks up
    # the static array, and torch's own kernels are loaded on their first use
    for t in outs:
        t.fill_(float("nan"))
    assert call() == N.OK
    torch.cuda.synchronize()
    [t.cpu() for t in outs]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for k in range(2):
        for t in outs:
            t.fill_(float("nan"))
        torch.cuda.synchronize()
        assert call() == N.OK, k
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free0, "the call took device memory"
        Om, Em, S, cR, cI = [t.cpu().numpy() for t in outs]
        assert relmax(Om, ref["O"]) < 1e-12
        assert abs(Em[0] - ref["energy"][0]) < 1e-12 * abs(ref["energy"][0])
        assert abs(Em[1] - ref["energy"][1]) < 1e-12 * max(abs(ref["energy"][1]), 1e-300) + 1e-300
        assert relmax(S.reshape(p, p), ref["S"]) < 1e-12
        assert relmax(cR, ref["cov_OER"]) < 1e-12
        assert relmax(cI, ref["cov_OEI"]) < 1e-12
    # sizes beyond the static array's limit are refused with an argument error
    code = lib.tdvmc_reduce_walkers_noalloc(C.c_void_p(O.data_ptr()), C.c_void_p(E.data_ptr()), nw, 33,
                                            *[C.c_void_p(t.data_ptr()) for t in outs], stream)
    assert code == N.ERR_ARG
    s.close()
