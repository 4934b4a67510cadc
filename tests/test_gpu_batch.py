"""Batched form against independent per-instance oracle runs: uneven sizes,
different materials and boundary codes, one stiff instance (relaxation time
far below the time step), per-instance CFL clocks."""
import numpy as np
import pytest
import torch

from conftest import rel_err
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _instances():
    from phd_gb300 import problems
    rng = np.random.default_rng(11)
    out = []
    sizes = [37, 128, 64, 200, 53, 96]
    for k, nx in enumerate(sizes):
        mu = [1e-2, 3e-3, 1e-1, 1e-2, 1e-4, 2e-2][k]
        cs = [1.0, 2.0, 0.7, 1.5, 5.0, 1.0][k]
        gamma = [1.4, 1.3, 1.67, 1.4, 1.25, 1.5][k]
        rhoL, rhoR = rng.uniform(0.2, 2.0, 2)
        pL, pR = np.exp(rng.uniform(np.log(0.2), np.log(5.0), 2))
        vL, vR = rng.uniform(-0.3, 0.3, 2)
        u, MP, tf, dX, bcs = problems.shock_tube(nx=nx, mu=mu, cs=cs, gamma=gamma, rhoL=rhoL,
                                                  pL=pL, rhoR=rhoR, pR=pR, vL=(vL, 0, 0),
                                                  vR=(vR, 0, 0))
        bc = "periodic" if k == 3 else "transitive"
        out.append((u, MP, dX, bc))
    return out


STIFF = 4  # relaxation time 2.4e-5, far below dt ~ 4e-4 .. 2e-3


def _oracle_step(O, u, MP, dX, bc, t, count):
    """One oracle step (timestep -> boundaries -> ADER -> renorm) from u."""
    nX = np.array([u.shape[0]], dtype=np.int32)
    code = 1 if bc == "periodic" else 0
    un = np.ascontiguousarray(u, dtype=np.float64).ravel().copy()
    dt = O.timestep(un, dX, 0.8, t, 0.2, count, MP)
    ub = O.boundaries(un, nX, np.array([code, code], dtype=np.int32))
    O.ader_stepper(un, ub, nX, dt, dX, MP)
    O.renorm_distortion(un, MP)
    return un.reshape(u.shape), dt


def test_batch_matches_oracle_every_step():
    """Per-step parity: after each batched step, every instance equals one
    oracle step taken from that instance's previous batched state."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from phd_gb300.batch import Batch
    insts = _instances()
    steps = 9  # crosses the first-five-steps dt reduction
    B = Batch(insts, cfl=0.8, tf=0.2)
    O = Oracle()
    newton_seen = False
    for s in range(steps):
        prev = [B.state(k).cpu().numpy().copy() for k in range(len(insts))]
        t_prev, _ = B.times()
        B.step(1)
        torch.cuda.synchronize()
        t_now, count = B.times()
        assert (count == s + 1).all()
        for k, (u0, MP, dX, bc) in enumerate(insts):
            ref, dt = _oracle_step(O, prev[k], MP, dX, bc, t_prev[k], s)
            assert abs((t_now[k] - t_prev[k]) - dt) <= 1e-12 * dt, (s, k)
            err = rel_err(B.state(k).cpu().numpy(), ref)
            assert err < 1e-10, (s, k, err)
        st = B.status.cpu().numpy()
        newton_seen |= bool(((st & 0xff) == 1).any())
        assert ((st & 0xff) != 2).all()
    assert newton_seen, "the stiff instance must exercise the Newton pass"
    # every instance advanced every step: updates = steps * sum(nx)
    assert int(B.updates.item()) == steps * int(B.nx.sum())


def test_batch_matches_independent_oracle_runs():
    """Whole-trajectory parity over nine steps for the non-stiff instances.
    The stiff instance is held to per-step parity only: the reference's
    Picard stopping rule (|dq| <= 6e-6 (1 + |q0|)) makes its predictor
    discontinuous in its input, so a 1e-12 difference that flips one cell's
    iteration count moves that step's result by ~1e-8, and later steps carry
    it."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from phd_gb300.batch import Batch
    insts = _instances()
    steps = 9
    B = Batch(insts, cfl=0.8, tf=0.2)
    B.step(steps)
    torch.cuda.synchronize()
    O = Oracle()
    t_gpu, count = B.times()
    assert (count == steps).all()
    for k, (u0, MP, dX, bc) in enumerate(insts):
        if k == STIFF:
            continue
        code = 1 if bc == "periodic" else 0
        ref, n, t = O.run(u0, MP, 0.2, dX, code, cfl=0.8, max_steps=steps)
        assert n == steps
        assert abs(t - t_gpu[k]) <= 1e-12 * t
        got = B.state(k).cpu().numpy()
        assert rel_err(got, ref) < 1e-8, (k, rel_err(got, ref))


def test_batch_equals_single_instance_path():
    """The batched kernels and the one-grid kernels give the same numbers for
    the same instance (the batched form changes indexing only)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from phd_gb300 import api
    from phd_gb300.batch import Batch
    from phd_gb300.driver import Stepper
    insts = _instances()
    B = Batch(insts, cfl=0.8, tf=0.2)
    for k in (0, STIFF):
        u0, MP, dX, bc = insts[k]
        nX = np.array([u0.shape[0]], dtype=np.int32)
        api.set_nvar(u0.shape[1])
        st = Stepper(nX, u0.shape[1])
        u = torch.tensor(u0.ravel(), device="cuda")
        t, count = 0.0, 0
        for _ in range(7):
            dt = float(api.timestep_device(u, dX, 0.8, t, 0.2, count, MP, out=st.dt).item())
            st.step(u, dt, dX, [0, 0], MP)
            t += dt
            count += 1
        if k == 0:
            B.step(7)
            torch.cuda.synchronize()
        err = rel_err(B.state(k).cpu().numpy().ravel(), u.cpu().numpy())
        # the stiff instance's Newton pass stops at |delta| <= 1e-11 (1 + |q|)
        # with FP32 corrections (contraction ~1e-2 per iteration), so its
        # result carries the last ~1e-13 of its inputs, which the two paths
        # round differently (the batch's autotuned face layout)
        assert err < (1e-12 if k == STIFF else 1e-13), (k, err)


def test_batch_graph_replay_equals_eager():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from phd_gb300.batch import Batch
    insts = _instances()
    A = Batch(insts)
    A.step(4)
    Bg = Batch(insts, autotune=False)
    Bg.set_shapes(A.shapes())  # the same launch shapes as A
    g = Bg.capture(1)
    for _ in range(4):
        g.replay()
    torch.cuda.synchronize()
    assert torch.equal(A.u, Bg.u)
    assert torch.equal(A.clock, Bg.clock)


def test_batch_finished_instances_stop():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from phd_gb300.batch import Batch
    insts = _instances()[:2]
    B = Batch(insts, cfl=0.8, tf=0.004)
    B.step(60)
    torch.cuda.synchronize()
    t, count = B.times()
    assert np.allclose(t, 0.004, rtol=0, atol=1e-15)
    O = Oracle()
    for k, (u0, MP, dX, bc) in enumerate(insts):
        ref, n, tt = O.run(u0, MP, 0.004, dX, 0, cfl=0.8)
        assert count[k] == n
        assert rel_err(B.state(k).cpu().numpy(), ref) < 1e-8


def test_batch_autotuner():
    """The autotuner times every candidate shape of each stage and keeps the
    fastest; a batch starts from the default shapes; every candidate gives
    the same step (the face pass's lane layout changes the order of a short
    sum: 1e-13), and invalid shapes are rejected."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from phd_gb300.batch import Batch
    insts = _instances()
    B = Batch(insts)
    sh = B.shapes()
    assert sh == B.tuning["shapes"]
    t = np.array(B.tuning["candidate_ms"])
    assert t.size == 22 and (t > 0).all()
    assert sh["weno_block"] == [64, 128, 256, 512][int(np.argmin(t[0:4]))]
    k = int(np.argmin(t[4:13]))
    assert (sh["first_block"], sh["picard_block"]) == ([32, 64, 128][k // 3], [32, 64, 128][k % 3])
    k = int(np.argmin(t[13:19]))
    assert (sh["faces_four_lanes"], sh["faces_block"]) == (k // 3, [32, 64, 128][k % 3])
    assert sh["cells_block"] == [32, 64, 128][int(np.argmin(t[19:22]))]
    # the clocks and states are untouched by tuning apart from the coming dt
    u0 = np.concatenate([np.asarray(i[0]).reshape(-1) for i in insts])
    assert np.array_equal(B.u.cpu().numpy(), u0)
    ref = Batch(insts, autotune=False)
    assert ref.shapes() == dict(zip(Batch.SHAPE_NAMES, [256, 128, 128, 0, 128, 128]))
    ref.step(3)
    B.step(3)
    torch.cuda.synchronize()
    base = ref.u.cpu().numpy()
    assert rel_err(B.u.cpu().numpy(), base) < 1e-13
    assert np.array_equal(B.clock.cpu().numpy(), ref.clock.cpu().numpy()) or \
        rel_err(B.clock.cpu().numpy(), ref.clock.cpu().numpy()) < 1e-13
    for split in (0, 1):
        for bs in (32, 64, 128):
            C = Batch(insts, autotune=False)
            C.set_shapes([64, bs, bs, split, bs, bs])
            C.step(3)
            torch.cuda.synchronize()
            assert rel_err(C.u.cpu().numpy(), base) < 1e-13, (split, bs)
    with pytest.raises(RuntimeError):
        C.set_shapes([64, 48, 128, 0, 128, 128])
    with pytest.raises(RuntimeError):
        C.set_shapes([64, 128, 128, 2, 128, 128])
