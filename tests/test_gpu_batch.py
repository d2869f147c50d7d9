"""Batched solves: every instance gives the same result alone and in the batch."""
import numpy as np
import pytest

import zisafvm_gb300 as z
from problems import polytrope_2d, vortex_2d

pytestmark = pytest.mark.gpu


def _single(mesh, scheme, u0, n_steps=0, t_end=0.0):
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    t, n = s.advance(n_steps=n_steps, t_end=t_end)
    u, _ = s.get_state()
    return u, t, n


@pytest.mark.parametrize("precision", [z.FP64, z.MIXED])
def test_batch_equals_alone(zlib, precision):
    probs = [polytrope_2d(n_rings=r, amplitude=a, seed=7 + r, precision=precision)
             for r, a in ((12, 1e-3), (20, 1e-2), (9, 1e-4))]
    raw, mesh, scheme, u0 = vortex_2d(n=16, halo=3)
    scheme.precision = precision
    probs.append((raw, mesh, scheme, u0))
    b = z.Batch(8)
    solvers, slots = [], []
    for k, (raw, mesh, scheme, u0) in enumerate(probs):
        s = z.Solver(mesh, scheme)
        s.set_state(u0)
        solvers.append(s)
        slots.append(b.add(s, n_steps=6 + 2 * k))
    for _ in range(10):
        if b.advance(4) == 0:
            break
    for k, (raw, mesh, scheme, u0) in enumerate(probs):
        st = b.status(slots[k])
        assert st["done"] and st["steps"] == 6 + 2 * k
        b.remove(slots[k])
        u_b, t_b = solvers[k].get_state()
        u_a, t_a, n_a = _single(mesh, scheme, u0, n_steps=6 + 2 * k)
        assert n_a == 6 + 2 * k
        if precision == z.FP64:
            # same FP64 arithmetic in the single and the batched kernels
            assert t_b == t_a
            assert np.array_equal(u_b, u_a), np.abs(u_b - u_a).max()
        else:
            # FP32 parts may be rounded differently by the two kernel builds
            assert abs(t_b - t_a) <= 1e-12 * t_a
            assert np.abs(u_b - u_a).max() <= 1e-10 * np.abs(u_a).max()


def test_batch_t_end(zlib):
    probs = [polytrope_2d(n_rings=r, amplitude=1e-3, seed=3, precision=z.MIXED) for r in (10, 16)]
    b = z.Batch(4)
    solvers, slots = [], []
    for (raw, mesh, scheme, u0), t_end in zip(probs, (0.01, 0.02)):
        s = z.Solver(mesh, scheme)
        s.set_state(u0)
        solvers.append(s)
        slots.append(b.add(s, t_end=t_end))
    while b.advance(8):
        pass
    for slot, t_end in zip(slots, (0.01, 0.02)):
        st = b.status(slot)
        assert st["done"] and abs(st["t"] - t_end) <= 1e-12 * t_end


def test_batch_autotune_keeps_results(zlib):
    """The launch shape the autotuner picks (cells or faces per tile = threads
    per block, 64 / 128 / 256, and the persistent grid) does not change results."""
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=14, amplitude=1e-3, precision=z.MIXED)
    s_tuned = z.Solver(mesh, scheme)
    s_tuned.set_state(u0)
    tuner = z.Batch(2)
    slot = tuner.add(s_tuned, n_steps=1000)
    assert tuner.tuned_shapes() == []  # no group before the first advance
    tuner.autotune(2)
    shapes = tuner.tuned_shapes()
    assert len(shapes) == 1 and shapes[0]["tuned"] and shapes[0]["block"] in (64, 128, 256), shapes
    tuner.remove(slot)
    u1, t1 = s_tuned.get_state()
    s_plain = z.Solver(mesh, scheme)
    s_plain.set_state(u1, t1)
    s_tuned.set_state(u1, t1)
    plain = z.Batch(2)
    a = tuner.add(s_tuned, n_steps=5)
    b = plain.add(s_plain, n_steps=5)
    while tuner.advance(4):
        pass
    while plain.advance(4):
        pass
    tuner.remove(a)
    plain.remove(b)
    x, _ = s_tuned.get_state()
    y, _ = s_plain.get_state()
    assert np.array_equal(x, y)


def test_batch_with_tracers_and_step_rejection(zlib):
    """Slots with advected variables and with step rejection, next to plain
    ones, give the single-solve results: FP64 bit for bit (cvars, avars, time
    and accepted steps)."""
    from problems import tracers
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=16, amplitude=1e-1)
    rej = z.Scheme(**{**scheme.__dict__, "step_rejection_drho": 2.4e-3, "step_rejection_max_exponent": 6})
    tr = z.Scheme(**{**scheme.__dict__, "n_avars": 2})
    both = z.Scheme(**{**rej.__dict__, "n_avars": 1})
    rawv, meshv, schv, uv = vortex_2d(n=16, halo=3)
    trv = z.Scheme(**{**schv.__dict__, "n_avars": 1})
    cases = [(mesh, scheme, u0, None), (mesh, rej, u0, None), (mesh, tr, u0, tracers(mesh, u0, 2)),
             (mesh, both, u0, tracers(mesh, u0, 1)), (meshv, trv, uv, tracers(meshv, uv, 1))]
    b = z.Batch(8)
    solvers, slots = [], []
    for m, sc, u, q in cases:
        s = z.Solver(m, sc)
        s.set_state(u)
        if q is not None:
            s.set_avars(q)
        solvers.append(s)
        slots.append(b.add(s, n_steps=12))
    for _ in range(20):
        if b.advance(4) == 0:
            break
    for k, (m, sc, u, q) in enumerate(cases):
        st = b.status(slots[k])
        assert st["done"] and st["steps"] == 12
        b.remove(slots[k])
        u_b, t_b = solvers[k].get_state()
        a = z.Solver(m, sc)
        a.set_state(u)
        if q is not None:
            a.set_avars(q)
        t_a, n_a = a.advance(n_steps=12)
        u_a, _ = a.get_state()
        assert n_a == 12 and t_b == t_a, (k, t_b, t_a)
        assert np.array_equal(u_b, u_a), (k, np.abs(u_b - u_a).max())
        if q is not None:
            assert np.array_equal(solvers[k].get_avars(), a.get_avars())
        if sc.step_rejection_drho > 0:
            assert a.step_rejections() > 0


def test_set_state_then_batch_advance(zlib):
    """A state uploaded into a solver that sits in a batch is what the next
    batch advance steps, even with no synchronisation in between (the batch
    stream waits for the solver's stream): every step uploads, advances the
    batch by one step and reads back, and matches the same sequence on a
    solver by itself, bit for bit in FP64."""
    probs = [polytrope_2d(n_rings=r, amplitude=1e-2, seed=r) for r in (20, 26)]
    b = z.Batch(4)
    solvers = []
    for raw, mesh, scheme, u0 in probs:
        s = z.Solver(mesh, scheme)
        s.set_state(u0)
        solvers.append(s)
        b.add(s, n_steps=1000)
    states = [u0.copy() for _, _, _, u0 in probs]
    for _ in range(4):
        for s, u in zip(solvers, states):
            s.set_state(u)
        b.advance(1)
        states = [s.get_state()[0] for s in solvers]
    for (raw, mesh, scheme, u0), u_b in zip(probs, states):
        a = z.Solver(mesh, scheme)
        u = u0.copy()
        for _ in range(4):
            a.set_state(u)
            a.advance(n_steps=1)
            u, _ = a.get_state()
        assert np.array_equal(u_b, u), np.abs(u_b - u).max()


def test_step_host_matches_separate_calls(zlib):
    """zfvm_step_host (upload, steps, download in one call) gives what
    set_state + advance + get_state give, for CFL steps and a fixed dt."""
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=20, amplitude=1e-2, seed=4)
    a = z.Solver(mesh, scheme)
    a.set_state(u0, 0.1)
    t_a, n_a = a.advance(n_steps=3)
    u_a, _ = a.get_state()
    b = z.Solver(mesh, scheme)
    u_b, t_b, n_b = b.step_host(u0, t=0.1, n_steps=3)
    assert (t_b, n_b) == (t_a, n_a) and np.array_equal(u_b, u_a)
    a.set_state(u0)
    a.step(1e-3)
    u_a, _ = a.get_state()
    out = u0.copy()
    u_b, t_b, n_b = b.step_host(out, n_steps=1, fixed_dt=1e-3, out=out)  # in place
    assert n_b == 1 and abs(t_b - 1e-3) < 1e-18 and np.array_equal(u_b, u_a)


def test_batch_advance_takes_exactly_the_steps_asked(zlib):
    """Batch.advance(n) replays n steps even when n is not a multiple of the
    captured step chunk (whole chunks, then a graph of the rest)."""
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=10, amplitude=1e-3, precision=z.MIXED)
    s = z.Solver(mesh, scheme)
    s.set_state(u0)
    b = z.Batch(1)
    slot = b.add(s, n_steps=1 << 40)
    total = 0
    for n in (12, 5, 8, 3):
        b.advance(n)
        total += n
        assert b.status(slot)["steps"] == total
    b.advance_timed(13)
    assert b.status(slot)["steps"] == total + 13


@pytest.mark.parametrize("precision", [z.FP64, z.MIXED])
def test_batch_step_host_matches_device_resident_steps(zlib, precision):
    """Batch.step_host (every slot's state in, one batched step, every state
    out, one host synchronisation) steps what a batch that keeps its states on
    the device steps: the states pass through the host in FP64, the FP32 pairs
    and the next step's CFL minimum are formed from them as the update forms
    them, so the states agree bit for bit, and the clocks count the same time
    and steps."""
    probs = [polytrope_2d(n_rings=r, amplitude=a, seed=r, precision=precision) for r, a in ((14, 1e-2), (22, 1e-4))]
    raw, mesh, scheme, u0 = vortex_2d(n=16, halo=3)
    scheme.precision = precision
    probs.append((raw, mesh, scheme, u0))

    def make():
        b = z.Batch(4)
        solvers, slots = [], []
        for raw, mesh, scheme, u0 in probs:
            s = z.Solver(mesh, scheme)
            s.set_state(u0)
            solvers.append(s)
            slots.append(b.add(s, n_steps=1000))
        return b, solvers, slots

    b1, s1, k1 = make()
    b1.advance(5)
    b2, s2, k2 = make()
    hosts = {k: u0.copy() for k, (_, _, _, u0) in zip(k2, probs)}
    for _ in range(5):
        assert b2.step_host(hosts, hosts, 1) == len(probs)
    for j in range(len(probs)):
        st1, st2 = b1.status(k1[j]), b2.status(k2[j])
        assert st1["steps"] == st2["steps"] == 5 and st1["t"] == st2["t"]
        u1, _ = s1[j].get_state()
        assert np.array_equal(hosts[k2[j]], u1), np.abs(hosts[k2[j]] - u1).max()
    # reading back only, and taking a state in without reading it back
    out = {k2[0]: np.zeros_like(hosts[k2[0]])}
    b2.step_host(None, out, 1)
    b1.advance(1)
    assert np.array_equal(out[k2[0]], s1[0].get_state()[0])
    b2.step_host({k2[1]: hosts[k2[1]]}, None, 1)
    with pytest.raises(z.ZfvmError):
        b2.step_host({k2[0]: np.zeros((3, 5))}, None, 1)


def test_batch_step_host_parts_groups_rejection_tracers(zlib):
    """The pipelined host round trip over more slots than parts, two kernel
    groups (FP64 and mixed), a periodic mesh, advected variables and step
    rejection: the same states, times and accepted steps as a batch that
    keeps its states on the device, FP64 and mixed bit for bit."""
    from problems import tracers
    raw, mesh, scheme, u0 = polytrope_2d(n_rings=16, amplitude=1e-1)
    rej = z.Scheme(**{**scheme.__dict__, "step_rejection_drho": 2.4e-3, "step_rejection_max_exponent": 6})
    tr = z.Scheme(**{**scheme.__dict__, "n_avars": 1})
    mix = z.Scheme(**{**scheme.__dict__, "precision": z.MIXED})
    mix_rej = z.Scheme(**{**rej.__dict__, "precision": z.MIXED})
    raw2, mesh2, sch2, u2 = polytrope_2d(n_rings=24, amplitude=1e-3, seed=5)
    rawv, meshv, schv, uv = vortex_2d(n=16, halo=3)
    cases = [(mesh, scheme, u0, None), (mesh, rej, u0, None), (mesh2, sch2, u2, None), (mesh, tr, u0, tracers(mesh, u0, 1)),
             (mesh, mix, u0, None), (mesh, mix_rej, u0, None), (meshv, schv, uv, None),
             (mesh2, z.Scheme(**{**sch2.__dict__, "precision": z.MIXED}), u2, None)]

    def make():
        b = z.Batch(len(cases))
        solvers, slots = [], []
        for m, sc, u, q in cases:
            s = z.Solver(m, sc)
            s.set_state(u)
            if q is not None:
                s.set_avars(q)
            solvers.append(s)
            slots.append(b.add(s, n_steps=1000))
        return b, solvers, slots

    n = 10
    b1, s1, k1 = make()
    b1.advance(n)
    b2, s2, k2 = make()
    hosts = {k: c[2].copy() for k, c in zip(k2, cases)}
    for _ in range(n):
        b2.step_host(hosts, hosts, 1)
    for j, (m, sc, u, q) in enumerate(cases):
        st1 = b1.status(k1[j])
        b1.remove(k1[j])  # closes the last step (puts back a rejected one)
        u1, t1 = s1[j].get_state()
        st2 = b2.status(k2[j])
        assert (st1["steps"], st1["t"]) == (st2["steps"], st2["t"]), (j, st1, st2)
        assert np.array_equal(hosts[k2[j]], u1), (j, np.abs(hosts[k2[j]] - u1).max())
        if q is not None:
            assert np.array_equal(s2[j].get_avars(), s1[j].get_avars())
    assert s1[1].step_rejections() > 0 and s1[5].step_rejections() > 0


def test_batch_step_host_several_steps_and_membership_changes(zlib):
    """Round trips of several steps (a chunk graph and a tail graph per part),
    with a slot removed and another added between them: every remaining slot
    ends where a batch that keeps its states on the device ends."""
    sizes = (10, 14, 18, 22, 12)
    probs = [polytrope_2d(n_rings=r, amplitude=1e-2, seed=r, precision=z.MIXED) for r in sizes]

    def make(k):
        raw, mesh, scheme, u0 = probs[k]
        s = z.Solver(mesh, scheme)
        s.set_state(u0)
        return s

    b1, b2 = z.Batch(8), z.Batch(8)
    s1 = {k: make(k) for k in range(4)}
    s2 = {k: make(k) for k in range(4)}
    k1 = {k: b1.add(s, n_steps=1000) for k, s in s1.items()}
    k2 = {k: b2.add(s, n_steps=1000) for k, s in s2.items()}
    hosts = {k2[k]: probs[k][3].copy() for k in range(4)}
    b1.advance(11)
    assert b2.step_host(hosts, hosts, 11) == 4
    # slot 1 leaves, instance 4 joins both batches
    b1.remove(k1[1])
    b2.remove(k2[1])
    del hosts[k2[1]]
    s1[4], s2[4] = make(4), make(4)
    k1[4] = b1.add(s1[4], n_steps=1000)
    k2[4] = b2.add(s2[4], n_steps=1000)
    hosts[k2[4]] = probs[4][3].copy()
    b1.advance(5)
    assert b2.step_host(hosts, hosts, 5) == 4
    for k in (0, 2, 3, 4):
        b1.remove(k1[k])
        u1, t1 = s1[k].get_state()
        st2 = b2.status(k2[k])
        assert st2["steps"] == (16 if k != 4 else 5), (k, st2)
        assert np.array_equal(hosts[k2[k]], u1), (k, np.abs(hosts[k2[k]] - u1).max())
