"""Batched monopole CTCS instances (persistent launch over a tile work-list)
against the CPU checker instance by instance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _instances(k, seed=3, nmin=40, nmax=150):
    from acoustic_petsc_gb300 import workloads

    return workloads.monopole_batch(k, seed=seed, nmin=nmin, nmax=nmax)


def _oracle_run(oracle, m, nsteps):
    cfg = oracle.MonoCfg()
    for f, _ in oracle.MonoCfg._fields_:
        if f != "it0":
            setattr(cfg, f, m[f])
    cfg.it0 = 0
    z = np.zeros((m["ny"], m["nx"]))
    return oracle.ctcs_monopole(cfg, z, z, nsteps)


def test_batch_vs_oracle(hype, oracle):
    inst = _instances(7)
    b = hype.BatchLeapfrog([hype.Monopole(**m) for m in inst], tile=(32, 32))
    b.step(65)
    for q, m in enumerate(inst):
        a, p = b.get(q)
        ao, po = _oracle_run(oracle, m, 65)
        assert np.abs(p - po).max() <= TOL * np.abs(po).max()
        assert np.abs(a - ao).max() <= TOL * np.abs(ao).max()


def test_graph_and_tiles_do_not_change_results(hype):
    inst = _instances(5, seed=11)
    res = []
    for tile, graph in [((32, 32), True), ((32, 32), False), ((128, 16), True), ((64, 64), False), ((0, 0), True)]:
        b = hype.BatchLeapfrog([hype.Monopole(**m) for m in inst], tile=tile)
        b.step(40, graph=graph)
        b.step(23, graph=graph)
        res.append([b.get(q)[1] for q in range(len(inst))])
        b.close()
    for r in res[1:]:
        for x, y in zip(res[0], r):
            assert np.array_equal(x, y)


def test_full_batch_workload_vs_oracle(hype, oracle):
    """the batched-acoustics workload at its full size: 256 instances with sides drawn
    log-uniformly in [64, 1024] (seed 7), one persistent launch per step, the step graph-captured;
    every instance after 150 steps against the checker's run of that instance alone."""
    inst = _instances(256, seed=7, nmin=64, nmax=1024)
    b = hype.BatchLeapfrog([hype.Monopole(**m) for m in inst])
    b.step(150)
    worst = 0.0
    for q, m in enumerate(inst):
        a, p = b.get(q)
        ao, po = _oracle_run(oracle, m, 150)
        worst = max(worst, np.abs(p - po).max() / np.abs(po).max(), np.abs(a - ao).max() / np.abs(ao).max())
    b.close()
    print(f"256 instances, 150 steps: worst relative L-inf {worst:.2e}")
    assert worst <= TOL


def test_size_classes_do_not_change_results(hype):
    """the size classes (own streams, launch priorities) touch disjoint parts of the level
    pools: any number of classes gives bit-identical instances"""
    inst = _instances(9, seed=13)
    res = []
    for ncls in (1, 0, 3, 9):
        b = hype.BatchLeapfrog([hype.Monopole(**m) for m in inst], tile=(32, 32))
        b.set_classes(ncls)
        b.step(47)
        b.step(31)
        res.append([b.get(q) for q in range(len(inst))])
        b.close()
    for r in res[1:]:
        for (a0, p0), (a1, p1) in zip(res[0], r):
            assert np.array_equal(a0, a1) and np.array_equal(p0, p1)


def test_instance_completion_times(hype):
    """each instance's completion time of a call: positive, equal within a class, and the
    smallest class (highest priority) done no later than the largest"""
    inst = _instances(24, seed=17, nmin=40, nmax=400)
    b = hype.BatchLeapfrog([hype.Monopole(**m) for m in inst], tile=(32, 32))
    b.set_classes(0)
    n, cls = b.classes()
    b.step(120)
    t = b.instance_times()
    assert n >= 1 and cls.min() == 0 and cls.max() == n - 1
    assert (t > 0).all()
    for c in range(n):
        assert np.ptp(t[cls == c]) == 0.0
    sizes = np.array([m["nx"] * m["ny"] for m in inst])
    assert sizes[cls == 0].max() <= sizes[cls == n - 1].min()
    assert t[cls == 0][0] <= t[cls == n - 1][0]
    print(f"{n} classes; completion times {sorted(set(np.round(t * 1e3, 3)))} ms")
    b.close()
