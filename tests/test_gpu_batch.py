"""Batched replicas: every replica of a mixed batch (dims, potential,
dynamics, precision, N) gives bit-identical results to the same replica run
alone in its own context, and the split-precision path meets its stated
error (force relative RMS <= 1e-5; NVE energy drift per particle, scaled to
1e5 steps, <= 1e-4)."""
import numpy as np
import pytest

from simulationcode_gb300 import _lib
from simulationcode_gb300.batch import ReplicaBatch
from simulationcode_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _mixed_specs(seed=0):
    rng = np.random.default_rng(seed)
    specs = [
        W.berthier_spec(700, 2, _lib.BROWNIAN, rng, dt=1e-4, precision=_lib.FP32_SPLIT, seed=11),
        W.berthier_spec(1500, 3, _lib.LANGEVIN, rng, dt=1e-3, precision=_lib.FP64, seed=12),
        W.lj_spec(1000, 3, _lib.NEWTONIAN, rng, dt=0.002, precision=_lib.FP32_SPLIT, seed=13),
        W.berthier_spec(2100, 3, _lib.BROWNIAN, rng, dt=1e-4, precision=_lib.FP64, seed=14),
        W.lj_spec(900, 2, _lib.LANGEVIN, rng, dt=0.002, precision=_lib.FP64, seed=15),
        W.berthier_spec(3000, 2, _lib.NEWTONIAN, rng, dt=1e-3, precision=_lib.FP32_SPLIT, seed=16),
    ]
    return specs


def _relaxed(specs):
    b = ReplicaBatch(0)
    ids = [b.add(s) for s in specs]
    b.rebuild()
    b.relax(300, 1e-3, 0.05)
    for i, s in zip(ids, specs):
        s.r = b.state(i)[0]
    b.close()
    return specs


def test_replica_alone_equals_in_the_mix(simlib):
    specs = _relaxed(_mixed_specs())
    mix = ReplicaBatch(0, graphs=True, graph_steps=8)
    ids = [mix.add(s) for s in specs]
    mix.rebuild()
    mix.step(37)
    for i, s in zip(ids, specs):
        alone = ReplicaBatch(0, graphs=False)
        a = alone.add(s)
        alone.rebuild()
        alone.step(37)
        for x, y in zip(alone.state(a), mix.state(i)):
            assert np.array_equal(x, y)
        assert alone.stats(a).rebuilds == mix.stats(i).rebuilds
        alone.close()
    mix.close()


def test_replicas_added_and_removed_between_steps(simlib):
    specs = _relaxed(_mixed_specs(seed=1))
    b = ReplicaBatch(0)
    first = [b.add(s) for s in specs[:3]]
    b.rebuild()
    b.step(10)
    b.remove(first[1])
    late = b.add(specs[3])
    b.step(10)
    ref = ReplicaBatch(0)
    a = ref.add(specs[3])
    ref.rebuild()
    ref.step(10)
    for x, y in zip(ref.state(a), b.state(late)):
        assert np.array_equal(x, y)
    b.close()
    ref.close()


def test_split_precision_nve_drift(simlib):
    rng = np.random.default_rng(3)
    s64 = W.berthier_spec(8000, 3, _lib.NEWTONIAN, rng, dt=0.005, precision=_lib.FP64, seed=21)
    (s64,) = _relaxed([s64])
    import copy
    s32 = copy.copy(s64)
    s32.precision = _lib.FP32_SPLIT
    out = {}
    for name, s in (("fp64", s64), ("fp32", s32)):
        b = ReplicaBatch(0)
        i = b.add(s)
        b.rebuild()
        b.step(2000)  # equilibrate off the relaxed start
        t, e = [], []
        for k in range(21):
            st = b.energies()[i]
            t.append(k * 200)
            e.append((st.epot + st.ekin) / s.N)
            b.step(200)
        slope = np.polyfit(np.array(t, float), np.array(e), 1)[0]
        out[name] = slope * 1e5  # energy per particle per 1e5 steps
        b.close()
    print("NVE drift per particle per 1e5 steps:", out)
    # the split-precision path adds no drift beyond the FP64 path's (the
    # reference arithmetic), within the 1e-4 per particle per 1e5 steps budget
    assert abs(out["fp32"]) <= abs(out["fp64"]) + 1e-4, out


@pytest.mark.parametrize("dims", [3, 2])
def test_split_precision_force_error_at_a_quench(simlib, dims):
    """Force relative RMS of the split path against FP64 on a relaxed start
    (capped steepest descent: pair forces near contact, net forces a
    partial cancellation of them -- the hardest state for FP32 pair
    arithmetic), inside the 1e-5 bar."""
    import copy
    from simulationcode_gb300 import precision
    rng = np.random.default_rng(7)
    s = W.berthier_spec(32768 if dims == 3 else 16384, dims, _lib.NEWTONIAN, rng, dt=0.005, precision=_lib.FP64,
                        seed=5)
    W.relax_on_device([s], 0, steps=300)
    rms, de = precision._forces_and_energy(s, 0, s.r)
    print("quench force relative RMS %.3e, |dE|/N %.3e" % (rms, de))
    assert rms <= 1e-5 and de <= 1e-6


def test_batched_host_transfers_equal_per_replica_calls(simlib):
    """simmd_upload_all / simmd_download_all (every replica in one call, the
    replicas' blocks in id order) give the same device state and the same
    host arrays as simmd_upload_r / simmd_download_r replica by replica, bit
    for bit, also after a replica has been removed (the layout closes up)."""
    specs = _relaxed(_mixed_specs(seed=3))
    a, b = ReplicaBatch(0), ReplicaBatch(0)
    ia = [a.add(s) for s in specs]
    ib = [b.add(s) for s in specs]
    for batch, ids in ((a, ia), (b, ib)):
        batch.rebuild()
        batch.step(5)
        batch.remove(ids[1])
    keep = [k for k in range(len(specs)) if k != 1]
    rng = np.random.default_rng(4)
    new = {k: (np.mod(specs[k].r + rng.uniform(-0.01, 0.01, specs[k].r.shape), specs[k].box_size),
               rng.standard_normal(specs[k].r.shape) * 0.3) for k in keep}
    # per replica on a
    for k in keep:
        s = specs[k]
        _lib.check(a.lib.simmd_upload_r(a.ctx, ia[k], _lib.ptr(new[k][0]), _lib.ptr(new[k][1]), None,
                                        _lib.ptr(np.ascontiguousarray(s.D)), None))
    # all at once on b
    total, offs = b.transfer_layout()
    assert sorted(offs) == [ib[k] for k in keep]
    r_all, v_all = np.zeros(total), np.zeros(total)
    D_all = np.concatenate([specs[k].D for k in keep])
    for k in keep:
        o, n = offs[ib[k]], specs[k].N * specs[k].dims
        r_all[o:o + n] = new[k][0].reshape(-1)
        v_all[o:o + n] = new[k][1].reshape(-1)
    assert total == sum(specs[k].N * specs[k].dims for k in keep)
    b.upload_all(r_all, D_all, v=v_all)
    for batch in (a, b):
        batch.step(23)
    r_o, v_o, F_o = np.zeros(total), np.zeros(total), np.zeros(total)
    b.download_all(r_o, v_o, F_o)
    for k in keep:
        o, n = offs[ib[k]], specs[k].N * specs[k].dims
        ra, va, Fa = a.state(ia[k])
        assert np.array_equal(ra.reshape(-1), r_o[o:o + n])
        assert np.array_equal(va.reshape(-1), v_o[o:o + n])
        assert np.array_equal(Fa.reshape(-1), F_o[o:o + n])
        assert a.stats(ia[k]).rebuilds == b.stats(ib[k]).rebuilds
    a.close()
    b.close()


def test_download_all_after_layout_query_and_skin_change(simlib):
    """simmd_download_all right after simmd_transfer_layout (no upload in
    between) and after a skin change: every replica's block equals its
    simmd_download_r copy (the device descriptors get the offsets that the
    layout query set on the host)."""
    specs = _relaxed(_mixed_specs(seed=5))
    b = ReplicaBatch(0)
    ids = [b.add(s) for s in specs]
    b.rebuild()
    b.step(4)

    def check():
        total, offs = b.transfer_layout()
        r = np.full(total, np.nan)
        b.download_all(r)
        for rid, s in zip(ids, specs):
            o, n = offs[rid], s.N * s.dims
            assert np.array_equal(b.state(rid)[0].reshape(-1), r[o:o + n]), rid

    check()
    b.set_skin(0.45, ids[2])
    b.step(3)
    check()
    b.close()


def test_set_state_all_equals_per_replica_set_state(simlib):
    """simmd_set_state_all (every replica in one call, lists and skin
    bookkeeping kept) equals simmd_set_state_r replica by replica, bit for
    bit; handing back the state just downloaded leaves the trajectory and the
    rebuild count as if the call had not been made (the segment loop of a
    caller that holds the state on the host)."""
    specs = _relaxed(_mixed_specs(seed=6))
    a, b, c = ReplicaBatch(0), ReplicaBatch(0), ReplicaBatch(0)
    ia = [a.add(s) for s in specs]
    ib = [b.add(s) for s in specs]
    ic = [c.add(s) for s in specs]
    for batch in (a, b, c):
        batch.rebuild()
        batch.step(9)
    # c: the state goes to the host and back between two segments
    total, offs = c.transfer_layout()
    r_h, v_h = np.zeros(total), np.zeros(total)
    c.download_all(r_h, v_h)
    c.set_state_all(r_h, v_h)
    rebuilds_before = [c.stats(i).rebuilds for i in ic]
    # a per replica, b at once: positions moved within the skin, new velocities
    rng = np.random.default_rng(7)
    new = {}
    for k, s in enumerate(specs):
        r0 = a.state(ia[k])[0]
        new[k] = (np.mod(r0 + rng.uniform(-0.004, 0.004, r0.shape), s.box_size), rng.standard_normal(r0.shape) * 0.3)
        _lib.check(a.lib.simmd_set_state_r(a.ctx, ia[k], _lib.ptr(new[k][0]), _lib.ptr(new[k][1]), None, None))
    total_b, offs_b = b.transfer_layout()
    r_all, v_all = np.zeros(total_b), np.zeros(total_b)
    for k, s in enumerate(specs):
        o, n = offs_b[ib[k]], s.N * s.dims
        r_all[o:o + n] = new[k][0].reshape(-1)
        v_all[o:o + n] = new[k][1].reshape(-1)
    b.set_state_all(r_all, v_all)
    for batch in (a, b, c):
        batch.step(21)
    ref = ReplicaBatch(0)
    ir = [ref.add(s) for s in specs]
    ref.rebuild()
    ref.step(30)
    for k in range(len(specs)):
        for x, y in zip(a.state(ia[k]), b.state(ib[k])):
            assert np.array_equal(x, y), k
        assert a.stats(ia[k]).rebuilds == b.stats(ib[k]).rebuilds
        for x, y in zip(ref.state(ir[k]), c.state(ic[k])):
            assert np.array_equal(x, y), k
        assert ref.stats(ir[k]).rebuilds == c.stats(ic[k]).rebuilds
        assert c.stats(ic[k]).rebuilds >= rebuilds_before[k]
    for batch in (a, b, c, ref):
        batch.close()


def test_deferred_replica_sums_equal_the_in_pass_reduction(simlib):
    """A batch of many small replicas leaves the stepping force pass's replica
    sums (mean force, centre-of-mass velocity) to a pass of their own, which
    adds the tiles' warp partials in the order of the in-pass tile reduction:
    every replica's trajectory equals its run alone (in-pass reduction) bit
    for bit, and the batch runs the extra pass each step."""
    import ctypes as C
    rng = np.random.default_rng(8)
    specs = []
    for k in range(200):
        dims = 2 if k % 2 else 3
        dyn = (_lib.BROWNIAN, _lib.LANGEVIN, _lib.NEWTONIAN)[k % 3]
        prec = _lib.FP32_SPLIT if k % 4 else _lib.FP64
        specs.append(W.berthier_spec(int(rng.integers(450, 600)), dims, dyn, rng, dt=1e-3, precision=prec,
                                     seed=100 + k))
    specs = _relaxed(specs)
    mix = ReplicaBatch(0, graphs=True, graph_steps=8)
    ids = [mix.add(s) for s in specs]
    mix.rebuild()
    f, rb = C.c_int64(), C.c_int64()
    assert simlib.simmd_kernel_counts(mix.ctx, C.byref(f), C.byref(rb)) == 0
    l0, rb0 = mix.launches(), rb.value
    mix.step(24)
    assert simlib.simmd_kernel_counts(mix.ctx, C.byref(f), C.byref(rb)) == 0
    # a step: kick1+drift and a rebuild plan (Newtonian/Langevin), the force
    # pass (one launch per precision), the replica sums, the position update
    # and a rebuild plan (Brownian); seven per rebuild body run; the closing
    # COM pass
    assert mix.launches() - l0 == 24 * (1 + 1 + 2 + 1 + 1 + 1) + 7 * (rb.value - rb0) + 1
    for k in (0, 1, 2, 3, 4, 5, 101, 199):
        alone = ReplicaBatch(0, graphs=False)
        a = alone.add(specs[k])
        alone.rebuild()
        alone.step(24)
        for x, y in zip(alone.state(a), mix.state(ids[k])):
            assert np.array_equal(x, y), k
        assert alone.stats(a).rebuilds == mix.stats(ids[k]).rebuilds
        alone.close()
    mix.close()
