"""Batched solves on the GPU: a problem gives the same bits alone, in a batch and in an ensemble.

No kernel reduces across slots, so batch composition must not change any result: the checks are
exact equality.  Accuracy of the batched path against the oracle is checked on one slot.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def state(mo, n, seed):
    return mo.random_spectrum_state(mo.Grid(n), seed).astype(np.complex64)


def alone(pkg, n, s0, nu, eta, dt, steps, stepper="RK4"):
    with pkg.Problem(pkg.GPU(0), nx=n, nu=nu, eta=eta, dt=dt, stepper=stepper) as p:
        p.set_sol(s0.T)
        pkg.stepforward(p, steps)
        return p.sol_c()


def test_batch_equals_alone_bitwise(pkg, mo):
    n, dt = 32, 0.2 * (2 * math.pi / 32)
    params = [(1e-3, 2e-3), (3e-3, 1e-3), (5e-4, 5e-4)]
    s0 = [state(mo, n, 40 + i) for i in range(3)]
    with pkg.Batch(n, capacity=4) as b:
        slots = [b.add(nu, eta, dt) for nu, eta in params]
        for s, x in zip(slots, s0):
            b.set_state(s, x)
        b.step(5)
        got = [b.get_state(s) for s in slots]
        for s in slots:
            assert b.clock(s)[1] == 5
    for i, (nu, eta) in enumerate(params):
        ref = alone(pkg, n, s0[i], nu, eta, dt, 5)
        assert np.array_equal(got[i], ref), i


def test_batch_membership_changes(pkg, mo):
    n, dt = 48, 0.2 * (2 * math.pi / 48)
    a0, b0, c0 = (state(mo, n, s) for s in (1, 2, 3))
    with pkg.Batch(n, capacity=3, stepper="LSRK4") as b:
        sa = b.add(1e-3, 1e-3, dt)
        sb = b.add(2e-3, 2e-3, dt)
        b.set_state(sa, a0)
        b.set_state(sb, b0)
        b.step(2)
        b.remove(sb)
        sc = b.add(4e-3, 1e-3, dt)  # reuses a free slot, state starts at zero
        assert np.all(b.get_state(sc) == 0)
        b.set_state(sc, c0)
        b.step(3)
        ga, gc = b.get_state(sa), b.get_state(sc)
        assert b.info() == (3, 2)
        assert b.clock(sa)[1] == 5 and b.clock(sc)[1] == 3
    assert np.array_equal(ga, alone(pkg, n, a0, 1e-3, 1e-3, dt, 5, "LSRK4"))
    assert np.array_equal(gc, alone(pkg, n, c0, 4e-3, 1e-3, dt, 3, "LSRK4"))


def test_ensemble_mixed_sizes(pkg, mo):
    cfg = {32: [(1e-3, 1e-3), (2e-3, 5e-4)], 64: [(5e-4, 1e-3)], 48: [(1e-3, 3e-3), (3e-3, 3e-3)]}
    batches, inits = {}, {}
    for n, ps in cfg.items():
        b = pkg.Batch(n, capacity=len(ps) + 1, stepper="LSRK4")
        dt = 0.2 * (2 * math.pi / n)
        for i, (nu, eta) in enumerate(ps):
            s = b.add(nu, eta, dt)
            x = state(mo, n, 100 * n + i)
            b.set_state(s, x)
            inits[(n, s)] = (x, nu, eta, dt)
        batches[n] = b
    ens = pkg.Ensemble(list(batches.values()))
    ens.step(4)
    ens.synchronize()
    got = {(n, s): batches[n].get_state(s) for (n, s) in inits}
    ens.close()
    for b in batches.values():
        b.close()
    for (n, s), (x, nu, eta, dt) in inits.items():
        assert np.array_equal(got[(n, s)], alone(pkg, n, x, nu, eta, dt, 4, "LSRK4")), (n, s)


def test_graph_and_direct_launches_agree(pkg, mo, lib):
    n, dt = 32, 1e-3
    x = state(mo, n, 9)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=dt) as p:
        p.set_sol(x.T)
        pkg.stepforward(p, 3)
        graph = p.sol_c()
        p.set_sol(x.T)
        pkg._lib.check(lib.mhd_profile_enable(p.handle, 1))
        pkg.stepforward(p, 3)
        pkg._lib.check(lib.mhd_profile_enable(p.handle, 0))
        direct = p.sol_c()
    assert np.array_equal(graph, direct)


def test_batch_slot_accuracy_vs_oracle(pkg, mo):
    n = 64
    g = mo.Grid(n)
    x = state(mo, n, 77)
    dt = 0.2 * (2 * math.pi / n)
    with pkg.Batch(n, capacity=2) as b:
        s = b.add(2e-3, 1e-3, dt)
        b.set_state(s, x)
        b.step(3)
        got = b.get_state(s)
        d = b.diagnostics(s)
    st = mo.Stepper(g, 2e-3, 1e-3, dt, "RK4", literal=False)
    ref = x.astype(np.complex128)
    for _ in range(3):
        st.stepforward(ref)
    g.dealias(ref)
    assert mo.rel_l2(got, ref, g.retained_mask()) < 2e-5
    assert d.nonfinite == 0 and d.max_divb < 1e-4
