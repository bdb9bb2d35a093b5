"""The learned contact-parameter guess: device training gradients against the
numpy reference, in-kernel inference against the training forward pass, and
what a trained network gains over the plain Newton start."""
import numpy as np
import pytest

from helpers import Pair, ellipsoids
from oracle import mlp_ref as M
from sucrose_gb300 import capi, mlp

pytestmark = pytest.mark.gpu
SIG = (3.0, 2.0, 1.0)


def small_ecp(counts=(8, 12, 16), seed=3):
    r, q, box = ellipsoids(counts, SIG, 0.1114, seed=seed, tilt=0.5)
    P = Pair(r, q, box, sig=SIG)
    P.g.init_nlist(0.3, 3.0, trigger_mode=1)
    return P


def test_mlp_gradients_match_reference(lib):
    import torch
    P = small_ecp()
    g = P.g
    capi.check(g.ctx, g.L.sg_mlp_init(g.ctx, 7))
    rng = np.random.default_rng(1)
    Xf = rng.normal(size=(512, 16)).astype(np.float32) * 0.7
    Xf[:, 14:] = 0.0
    y = rng.uniform(0.2, 0.8, size=512).astype(np.float32)
    X = torch.tensor(Xf, device="cuda").to(torch.bfloat16)
    yt = torch.tensor(y, device="cuda")
    gd, loss = mlp.grad(g, X, yt)
    w = g.get_mlp_weights()
    lref, gref, _ = M.forward_backward(w, X.float().cpu().numpy(), y.astype(np.float64), bf=True)
    assert abs(loss - lref) <= 1e-5 * abs(lref)
    blocks = [(M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
              (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.OFF_W4), (M.OFF_W4, M.OFF_B4), (M.OFF_B4, M.NPARAM)]
    for a, b in blocks:
        e = np.linalg.norm(gd[a:b] - gref[a:b]) / max(np.linalg.norm(gref[a:b]), 1e-30)
        # BF16 rounding of intermediate gradients may round differently when
        # their FP32 inputs differ in the last bit: 1e-2 norm-wise per block
        assert e < 1e-2, (a, b, e)


def test_inference_kernel_matches_training_forward(lib):
    import torch
    P = small_ecp(seed=4)
    g = P.g
    capi.check(g.ctx, g.L.sg_mlp_init(g.ctx, 11))
    g.zero_forces()
    g.pair_forces(g.params(capi.ECPR, solver=capi.SOLVER_NEWTON))
    k = g.npairs()
    X = torch.empty((k, 16), dtype=torch.bfloat16, device="cuda")
    y = torch.empty(k, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    import ctypes as C
    cnt = C.c_int64(0)
    capi.check(g.ctx, g.L.sg_mlp_features(g.ctx, C.c_void_p(X.data_ptr()), C.c_void_p(y.data_ptr()), k, C.byref(cnt)))
    assert cnt.value == k
    pred = mlp.predict(g, X).clamp(0.02, 0.98).cpu().numpy()
    inf = mlp.guess(g).cpu().numpy()
    assert np.max(np.abs(pred - inf)) < 2e-3


def test_features_refused_after_support_filtered_call(lib):
    """The support-filtered launch leaves lambda unset for the pairs it does
    not solve: collecting training samples after it is refused, and works
    again after a call that solves every pair."""
    import ctypes as C
    import torch
    P = small_ecp(seed=5)
    g = P.g
    p = g.params(capi.ECPR, solver=capi.SOLVER_NEWTON)
    k = g.npairs()
    X = torch.empty((k, 16), dtype=torch.bfloat16, device="cuda")
    y = torch.empty(k, dtype=torch.float32, device="cuda")
    cnt = C.c_int64(0)
    feats = lambda: g.L.sg_mlp_features(g.ctx, C.c_void_p(X.data_ptr()), C.c_void_p(y.data_ptr()), k,
                                        C.byref(cnt))
    g.set_launch(capi.ECPR, 256, 2)
    g.zero_forces()
    g.pair_forces(p)
    assert np.isnan(g.ecp_lambda()).any()
    assert feats() == capi.SG_ENOTREADY
    g.set_launch(capi.ECPR, 256, 0)
    g.zero_forces()
    g.pair_forces(p)
    assert feats() == capi.SG_OK and cnt.value == k
    assert not np.isnan(y.cpu().numpy()).any()


def test_tensor_core_guess_matches_warp_mma_guess(lib):
    """tcgen05 pass (TMEM accumulators) against the warp-level mma.sync path and
    the training forward: the same BF16 operands and FP32 accumulation, so the
    guesses agree to BF16 rounding of the hidden layers."""
    import torch
    P = small_ecp(seed=6)
    g = P.g
    capi.check(g.ctx, g.L.sg_mlp_init(g.ctx, 13))
    g.zero_forces()
    g.pair_forces(g.params(capi.ECPR, solver=capi.SOLVER_NEWTON))
    warp = mlp.guess(g).cpu().numpy()
    tc = mlp.guess_tc(g).cpu().numpy()
    assert tc.shape == warp.shape and np.all(np.isfinite(tc))
    assert np.max(np.abs(tc - warp)) < 2e-3


def test_tensor_core_wait_timeout_is_reported(lib):
    """A completion wait that runs out (the test hook issues no MMA) stops the
    pass with a status the host reads; the context stays usable."""
    P = small_ecp(seed=8)
    g = P.g
    capi.check(g.ctx, g.L.sg_mlp_init(g.ctx, 19))
    g.zero_forces()
    g.pair_forces(g.params(capi.ECPR, solver=capi.SOLVER_NEWTON))
    capi.check(g.ctx, g.L.sg_mlp_test_wait_timeout(g.ctx))
    with pytest.raises(capi.SgError) as e:
        mlp.guess_tc(g)
    assert e.value.code == capi.SG_ECUDA
    capi.check(g.ctx, g.L.sg_mlp_clear_error(g.ctx))
    ok = mlp.guess_tc(g).cpu().numpy()          # next pass runs normally
    assert np.all(np.isfinite(ok)) and np.max(np.abs(ok - mlp.guess(g).cpu().numpy())) < 2e-3


@pytest.mark.parametrize("inline", [0, 1])
def test_learned_guess_forces_match_fp64(lib, inline):
    """Forces of the learned-guess path (either inference path) against the
    FP64 oracle with the tightly converged contact parameter."""
    import oracle as O
    from helpers import rel
    P = small_ecp(seed=7)
    g = P.g
    capi.check(g.ctx, g.L.sg_mlp_init(g.ctx, 17))
    capi.check(g.ctx, g.L.sg_mlp_set_inline(g.ctx, inline))
    g.zero_forces()
    _, _, st = g.pair_forces(g.params(capi.ECPR, cutoff=3.0, solver=capi.SOLVER_MLP_NEWTON), want_stats=True)
    F, T = g.forces()
    assert st.nonconverged == 0
    pi, pj = P.o.pairs(3.0, 0.3)
    P.o.zero_forces()
    P.o.forces(O.pair_params(O.ECPR, cutoff=3.0, solver=O.SOLVER_TIGHT), pi, pj)
    Fo, To = P.oracle_forces()
    assert rel(F, Fo) < 1e-5 and rel(T, To) < 1e-5


def test_trained_guess_cuts_newton_iterations(lib):
    P = small_ecp(counts=(12, 16, 24), seed=5)
    g = P.g
    newton = g.params(capi.ECPR, solver=capi.SOLVER_NEWTON)

    def langevin(T):
        g.configure_step(newton, integrator=capi.INT_LANGEVIN, dt=0.001, target_temp=T, damping=1.0, rotations=1)

    X, y = mlp.generate(g, newton, langevin, samples=400_000, every=20, equil=100)
    hist = mlp.train(g, X, y, epochs=12, batch=8192, lr=3e-3, seed=2)
    assert hist[-1] < 0.2 * hist[0]
    g.zero_forces()
    _, _, plain = g.pair_forces(newton, want_stats=True)
    g.zero_forces()
    _, _, learned = g.pair_forces(g.params(capi.ECPR, solver=capi.SOLVER_MLP_NEWTON), want_stats=True)
    mean_plain = plain.solver_evals / plain.pairs
    mean_mlp = learned.solver_evals / learned.pairs
    print(f"Newton evaluations per pair: plain {mean_plain:.3f}, learned guess {mean_mlp:.3f}, "
          f"fallbacks {learned.fallbacks / learned.pairs:.4f}, final mse {hist[-1]:.2e}")
    assert learned.nonconverged == 0
    assert mean_mlp < mean_plain
    assert learned.fallbacks < 0.01 * learned.pairs
