"""simmd_energy_virial_noalloc -- the entry point for callers that cannot
allocate device memory (their GPU memory belongs to another pool or budget,
or their loop cannot afford an allocation) -- checked through the C ABI on
two calls in a row (the second call reuses the library's fixed scratch
array left over from the first):
  * against the oracle's calculate_full_energy and virial on the same
    positions and list, and against simmd_energy (the context path);
  * the second call reserves no device memory: free device memory
    (cudaMemGetInfo) and the torch allocator's reserved bytes are the same
    before and after it.

Tolerance: relative 1e-12 on energy and virial, as the other FP64 energy
tests.  Collected last (file name) so a stop-at-first-failure run has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from cases import make_case
from gpu_helpers import GpuSystem, to_simmd

pytestmark = pytest.mark.gpu


def _vp(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("pot,dims,N", [(1, 3, 1728), (0, 3, 1000), (1, 2, 1600), (0, 2, 900)])
def test_noalloc_energy_virial_matches_simmd_energy(simlib, oracle, pot, dims, N):
    torch = pytest.importorskip("torch")
    p, r, v, D, rc = make_case(pot, dims, 0, N, seed=21)
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc, full_list=True)
    gpu.rebuild()
    e_ref, w_ref, _ = gpu.energy()
    # the full neighbour list in the reference layout (maxK, N) column-major,
    # 1-based, placed in device memory owned by the caller (torch here)
    maxK = 200
    counts = np.zeros(N, np.int64)
    lst = np.zeros((N, maxK), np.int64)
    assert simlib.simmd_export_pairs(gpu.ctx, 1, maxK, C.c_void_p(counts.ctypes.data),
                                     C.c_void_p(lst.ctypes.data)) == 0
    r_now = gpu.state()[0]
    ref = oracle.OracleSystem(p, r_now, D, force_cutoff=rc)
    ref.update_neighbor_lists()
    e_orc, w_orc = ref.full_energy(), ref.virial()
    dev = torch.device("cuda:0")
    rd = torch.from_numpy(np.ascontiguousarray(r_now)).to(dev)
    Dd = torch.from_numpy(np.ascontiguousarray(D, dtype=np.float64)).to(dev)
    cd = torch.from_numpy(counts).to(dev)
    ld = torch.from_numpy(lst).to(dev)
    out = torch.zeros(3, dtype=torch.float64, device=dev)
    prm = to_simmd(p, force_cutoff=rc)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        free0, reserved0 = torch.cuda.mem_get_info(dev)[0], torch.cuda.memory_reserved(dev)
        st = simlib.simmd_energy_virial_noalloc(C.byref(prm), _vp(rd), _vp(Dd), _vp(cd), _vp(ld), maxK, _vp(out),
                                                stream)
        assert st == 0, simlib.simmd_status_string(st)
        torch.cuda.synchronize()
        free1, reserved1 = torch.cuda.mem_get_info(dev)[0], torch.cuda.memory_reserved(dev)
        if call == 1:  # the first call may load the library's device code
            assert free1 == free0 and reserved1 == reserved0
        e, w, bad = out.cpu().tolist()
        assert bad == 0.0
        assert e == pytest.approx(e_orc, rel=1e-12), call
        assert w == pytest.approx(w_orc, rel=1e-12), call
        assert e == pytest.approx(e_ref, rel=1e-12), call
        assert w == pytest.approx(w_ref, rel=1e-12), call
    gpu.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(simlib, oracle):
    torch = pytest.importorskip("torch")
    from simulationcode_gb300 import _lib
    p, r, v, D, rc = make_case(0, 3, 0, 1000, seed=1)
    prm = to_simmd(p, force_cutoff=rc)
    prm.N = 1048576 + 1  # SIMMD_NOALLOC_MAX_N + 1
    t = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    st = simlib.simmd_energy_virial_noalloc(C.byref(prm), _vp(t), _vp(t), _vp(t), _vp(t), 1, _vp(t), None)
    assert st == _lib.ERR_BUDGET
