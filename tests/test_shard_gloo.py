"""Multi-process sharding on CPU (gloo, world size 2): each rank integrates
its own particle range with the CPU oracle; the union of the ranks' results
equals a single-process run of all particles bit for bit, and the combined
timing/step figures are the maximum and the sum."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _problem():
    from particles_gb300 import fields, params
    qom, vun = 200.0, 1.0 / 20.0
    tmax = 0.5 * 2.0 * np.pi / qom
    prm = params.pack_params(qom=qom, vunit=vun, tmax=tmax, dtmax=tmax, atol=1e-8, rtol=1e-8)
    tg = params.time_grid(4, tmax)
    uu, bb = fields.snapshot(8, seed=5)
    return prm, tg, uu, bb


def _states(idx, tg):
    from particles_gb300 import initial
    st = np.zeros((idx.size, tg.size, 8))
    st[:, 0, :6] = initial.isotropic_state(idx.size, 5, speed=0.5, index=idx)
    return st


def _strong_states(n, tg):
    """A fixed particle set with gamma spread over two decades."""
    from particles_gb300 import initial
    st = np.zeros((n, tg.size, 8))
    st[:, 0, :6] = initial.isotropic_state(n, 7, gamma_range=(1.01, 100.0))
    return st


def _rank(rank, world, port, per_rank, out_dir, strong=False):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from particles_gb300.shard import combine, expected_work, particle_indices, weighted_ranges
    prm, tg, uu, bb = _problem()
    if strong:                       # one fixed set, ranges of equal expected work
        st = _strong_states(world * per_rank, tg)
        lo, hi = weighted_ranges(expected_work(st[:, 0, :6]), world)[rank]
        st = st[lo:hi].copy()
    else:
        st = _states(particle_indices(rank, per_rank), tg)
    s, c, _ = oracle.integrate("rk5", prm, tg, uu, bb, st, nthreads=1)
    t, a = combine(torch, 1.0 + rank, float(c[:, 1].sum()))
    parts = [None] * world
    torch.distributed.all_gather_object(parts, (s, c))
    if rank == 0:
        np.savez(os.path.join(out_dir, "out.npz"), s=np.concatenate([p[0] for p in parts]),
                 c=np.concatenate([p[1] for p in parts]), t=t, a=a)
    torch.distributed.barrier()
    torch.distributed.destroy_process_group()


def test_two_rank_sharding_matches_one_process(tmp_path, oracle_lib):
    import oracle
    mp = torch.multiprocessing.get_context("spawn")
    per_rank, world = 24, 2
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, world, port, per_rank, str(tmp_path)))
             for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    out = np.load(tmp_path / "out.npz")
    prm, tg, uu, bb = _problem()
    idx = np.arange(world * per_rank, dtype=np.uint64)
    s, c, _ = oracle.integrate("rk5", prm, tg, uu, bb, _states(idx, tg))
    assert np.array_equal(out["s"], s) and np.array_equal(out["c"], c)
    assert float(out["t"]) == 2.0                       # the slowest rank's time
    assert float(out["a"]) == float(c[:, 1].sum())      # the steps of all ranks


def test_two_rank_strong_scaling_weighted_ranges(tmp_path, oracle_lib):
    """One fixed particle set split by weighted_ranges (equal expected work
    by 1 / gamma): the concatenated ranges equal the one-process run, and the
    heavy low-gamma particles are not all on one rank."""
    import oracle
    from particles_gb300.shard import expected_work, weighted_ranges
    mp = torch.multiprocessing.get_context("spawn")
    per_rank, world = 24, 2
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, world, port, per_rank, str(tmp_path), True))
             for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    out = np.load(tmp_path / "out.npz")
    prm, tg, uu, bb = _problem()
    st = _strong_states(world * per_rank, tg)
    s, c, _ = oracle.integrate("rk5", prm, tg, uu, bb, st.copy())
    assert np.array_equal(out["s"], s) and np.array_equal(out["c"], c)
    w = expected_work(st[:, 0, :6])
    parts = [w[lo:hi].sum() for lo, hi in weighted_ranges(w, world)]
    assert max(parts) - min(parts) <= w.max()


def test_weighted_ranges_cover_and_balance():
    from particles_gb300.shard import weighted_ranges
    rng = np.random.default_rng(3)
    for n, world in ((1000, 4), (7, 3), (3, 8), (1, 1)):
        w = rng.uniform(0, 1, n) ** 8
        r = weighted_ranges(w, world)
        assert len(r) == world and r[0][0] == 0 and r[-1][1] == n
        assert all(a <= b for a, b in r) and all(r[i][1] == r[i + 1][0] for i in range(world - 1))
        sums = [w[a:b].sum() for a, b in r]
        assert max(sums) - w.sum() / world <= w.max() + 1e-12
    with pytest.raises(ValueError):
        weighted_ranges(np.array([1.0, -1.0]), 2)
