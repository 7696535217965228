"""The allocation-free evolver (song2_gpu_evolve_noalloc) against the regular
C-ABI path.

Some callers cannot allocate device memory: applications whose GPU memory
belongs to a fixed pool or to another runtime, and services that forbid
cudaMalloc after start-up.  The allocation-free entry point serves them by
keeping all its scratch in a fixed array compiled into the library; this test
checks, through the C ABI, that two calls in a row give the same sources as the
regular entry point, within the tolerance of the other parity tests, and that
every triplet's stats land in its slot of the reference work order (the same
step counts as the regular entry's).  The test allocates the input and output
buffers itself, as such a caller would have them from its own pool.
"""
import ctypes as C

import numpy as np
import pytest

from song_gb300 import capi
from helpers import floored_errors, gpu_run, problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kw", [
    dict(),
    # the delta-tilde coupling table is carved from the scratch too
    dict(sources="TEB", l_max=5, use_delta_tilde_in_los=1, rescale_cmb_sources=1, radiation_streaming_approximation=1),
])
def test_noalloc_matches_regular_entry_twice(lib, kw):
    torch = pytest.importorskip("torch")
    import oracle
    p = problem(**kw)
    p.set_first_order(oracle.first_order(p, nthreads=4))
    ref, st_ref, _ = gpu_run(lib, p, capi.SONG2_PREC_MIXED)
    # device copies of the tables (the caller's own buffers)
    dev = {name: torch.from_numpy(np.ascontiguousarray(getattr(p, name))).cuda()
           for name in ("bg", "bg_dd", "fo", "fo_dd")}
    tab = capi.Tables.from_buffer_copy(p.tables)
    for name, t in dev.items():
        setattr(tab, name, C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double)))
    src = torch.zeros(p.tp2_size * p.per_type, dtype=torch.float64, device="cuda")
    stats = torch.zeros(p.n_triplets * C.sizeof(capi.TripletStats) // 4, dtype=torch.int32, device="cuda")
    err = capi.errbuf()
    for call in range(2):
        src.fill_(float("nan"))     # the call must overwrite (and clear) the whole buffer
        rc = lib.song2_gpu_evolve_noalloc(C.byref(p.spec), C.byref(tab), capi.SONG2_PREC_MIXED,
                                          C.c_void_p(src.data_ptr()), C.c_void_p(stats.data_ptr()), None, err)
        assert rc == 0, err.value
        torch.cuda.synchronize()
        got = src.cpu().numpy()
        st = stats.view(-1, C.sizeof(capi.TripletStats) // 4).cpu().numpy()
        assert np.all(st[:, 0] == capi.SONG2_OK)
        # stats in the reference work order: each triplet's step count is the regular run's
        assert np.array_equal(st[:, 1], st_ref["n_steps"]), call
        assert np.max(floored_errors(got, ref, p)) < 10 * p.spec.rtol, call
