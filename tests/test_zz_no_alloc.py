"""The allocation-free VMC entry point (mole_vmc_run_noalloc) against the
regular one (mole_vmc_run).

mole_vmc_run_noalloc serves callers that cannot allocate device memory while
they run -- a host framework that owns every device buffer through its own
pool, or a loop that must not take cudaMalloc's implicit synchronisation --
so the caller passes all inputs and outputs as device memory and the library
works only in its fixed 2 MiB scratch array. Here PyTorch owns the caller's
buffers. Two calls in a row must reproduce the regular entry point's
trajectory, energy, blocking and SR sums on the same random streams, in
three launch shapes: 4,096 walkers in FP64 with SR sums (64-walker CTAs),
40,000 walkers in FP64 (a whole wave of CTAs with the walkers split evenly;
the regular entry point runs these through its packed-FP64 kernel, so the two
kernels are checked against each other too) and 4,096 walkers in the mixed
FP32-evaluation form with SR sums.

This file is collected last so that a failure here stops a -x run only after
every other test has run; it creates its own context and passes alone.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def _rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), 1.0)))


@pytest.mark.parametrize("W,prec,sr", [(4096, "fp64", True), (40000, "fp64", False), (4096, "mixed", True)])
def test_noalloc_matches_regular_entry_point_twice(W, prec, sr):
    torch = pytest.importorskip("torch")
    from mole_gb300 import _lib, api
    from mole_gb300 import system as S

    lib = _lib.load()
    ctx = api.Context(0)
    s = S.h2(1.0, 0.5)
    wf = api.WaveFunction(ctx, s)
    N, P = s.n_elec, s.n_params
    precision = {"fp64": api.PREC_FP64, "mixed": api.PREC_MIXED}[prec]
    seed = 0x5EED + W
    walkers = api.Walkers(wf, W, seed=seed)
    pos0 = walkers.positions()  # [W][N][3]

    dev = torch.device("cuda", 0)
    d_pos = torch.from_numpy(np.ascontiguousarray(pos0.reshape(W, 3 * N).T)).to(dev)  # SoA [3N][W]
    n_eq, n_steps, bs = 10, 60, 10
    d_mom = torch.zeros(_lib.NMOM, dtype=torch.float64, device=dev)
    d_tb = torch.zeros(n_steps // bs, dtype=torch.float64, device=dev)
    d_sr = torch.zeros(2 * P + P * P, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    sampler = api.Sampler(wf, api.MetropolisGaussian(0.4), walkers, precision=precision)
    step0 = 0
    for call in range(2):
        ref = sampler.run(n_eq, n_steps, bs, sr=sr)
        o = _lib.VmcOpts(S.MOVE_GAUSS, 0.4, n_eq, n_steps, bs, int(sr), precision, 0)
        rc = lib.mole_vmc_run_noalloc(wf.h, C.c_void_p(d_pos.data_ptr()), W, seed, step0, C.byref(o),
                                      C.c_void_p(d_mom.data_ptr()), C.c_void_p(d_tb.data_ptr()),
                                      C.c_void_p(d_sr.data_ptr()) if sr else None,
                                      C.c_void_p(stream.cuda_stream))
        _lib.check(rc)
        step0 += n_eq + n_steps
        torch.cuda.synchronize()
        mom = d_mom.cpu().numpy()
        pos = d_pos.cpu().numpy().T.reshape(W, N, 3)
        assert _rel(pos, walkers.positions()) < RTOL, call
        assert np.array_equal(mom[[0, 4, 5, 6]], ref.moments[[0, 4, 5, 6]]), call
        assert _rel(mom[1:4], ref.moments[1:4]) < RTOL, call
        assert _rel(d_tb.cpu().numpy(), ref.time_blocks) < RTOL, call
        if sr:
            srv = d_sr.cpu().numpy()
            assert _rel(srv[:P], ref.sum_O) < RTOL and _rel(srv[P:2 * P], ref.sum_EO) < RTOL, call
            assert _rel(srv[2 * P:].reshape(P, P), ref.sum_OO) < RTOL, call
        assert torch.cuda.current_device() == 0

    # sizes beyond the fixed scratch are rejected with a clear error
    big = _lib.VmcOpts(S.MOVE_GAUSS, 0.4, 0, 5000, 1, 0, api.PREC_FP64, 0)
    rc = lib.mole_vmc_run_noalloc(wf.h, C.c_void_p(d_pos.data_ptr()), W, seed, step0, C.byref(big),
                                  C.c_void_p(d_mom.data_ptr()), C.c_void_p(d_tb.data_ptr()), None,
                                  C.c_void_p(stream.cuda_stream))
    assert rc == 2 and b"scratch" in lib.mole_last_error_string()
    walkers.close()
    wf.close()
    ctx.close()
