"""Warm-start MLP: the CPU oracle pinned on its own (BF16 rounding against torch, backward
against finite differences), then the GPU kernels against the oracle: tensor-core inference,
FP32 loss/gradient, on-device training, and the warm-start plumbing inside the VBD solver."""
import numpy as np
import pytest

from oracle import mlp_ref as M

N = pytest.importorskip("spg_gb300.native")


def _weights(rng, scale=1.0):
    p = {}
    for name, shape in M.SHAPES:
        if name.startswith("W"):
            p[name] = rng.uniform(-1, 1, shape) * np.sqrt(6.0 / sum(shape)) * scale
        else:
            p[name] = rng.normal(scale=0.1, size=shape)
    return M.pack(p).astype(np.float32)


def _features(rng, n):
    x = rng.normal(size=(n, 24)).astype(np.float32)
    x[:, :15] *= 5.0          # scaled displacement histories span a few tens
    x[:, 18] = rng.random(n) < 0.1
    x[:, 23] = 1.0
    return x


# ----------------------------------------------------------------------------- CPU oracle


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    a = (rng.standard_normal(200000) * 10.0 ** rng.uniform(-8, 8, 200000)).astype(np.float32)
    ref = torch.from_numpy(a).to(torch.bfloat16).float().numpy()
    assert np.array_equal(ref, M.bf16_round(a))


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    w = rng.standard_normal(M.N_PARAMS) * 0.1
    x = rng.standard_normal((9, 24))
    t = rng.standard_normal((9, 3))
    _, g = M.loss_grad(w, x, t, quantize=False)
    idx = np.concatenate([rng.choice(M.N_PARAMS, 60, replace=False), [0, M.N_PARAMS - 1]])
    for i in idx:
        e = np.zeros_like(w)
        e[i] = 1e-6
        fd = (M.loss_grad(w + e, x, t, False)[0] - M.loss_grad(w - e, x, t, False)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, np.abs(g).max()), (i, fd, g[i])


def test_parameter_layout():
    assert M.N_PARAMS == 24 * 128 + 128 + 2 * (128 * 128 + 128) + 128 * 3 + 3 == 36611


# ----------------------------------------------------------------------------- GPU


@pytest.mark.gpu
def test_num_params_matches_oracle():
    assert N.Mlp.num_params() == M.N_PARAMS


@pytest.mark.gpu
def test_loss_gradient_matches_oracle():
    """Device forward/backward (tensor-core GEMMs with BF16 operands, FP32 accumulation) against
    the FP64 oracle with the same BF16 roundings of the weights and of every GEMM operand:
    gradient within 2e-3 of its largest entry per weight block (FP32 accumulation order, and an
    operand whose FP32 value sits next to a BF16 rounding boundary rounding the other way), and
    within 3e-2 of the unrounded FP64 gradient."""
    rng = np.random.default_rng(2)
    mlp = N.Mlp(seed=3)
    w = _weights(rng)
    mlp.set_weights(w)
    assert np.array_equal(mlp.weights(), w)
    x = _features(rng, 3000)
    t = rng.normal(size=(3000, 3)).astype(np.float32)
    loss, g = mlp.loss_grad(x, t)
    loss_ref, g_ref = M.loss_grad(w, x, t, emulate_bf16_operands=True)
    _, g_full = M.loss_grad(w, x, t)
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref
    o = 0
    for name, shape in M.SHAPES:
        n = int(np.prod(shape))
        a, b, c = g[o:o + n], g_ref[o:o + n], g_full[o:o + n]
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        print(f"{name}: max |g - g_bf16| / max |g_bf16| = {err:.2e}, against unrounded "
              f"{np.max(np.abs(a - c)) / np.max(np.abs(c)):.2e}")
        assert err <= 2e-3, name
        assert np.max(np.abs(a - c)) <= 3e-2 * np.max(np.abs(c)), name
        o += n


@pytest.mark.gpu
def test_tensor_core_inference_matches_oracle():
    """tcgen05 BF16 inference (FP32 accumulator in tensor memory) against the oracle evaluated
    with the kernel's BF16 operand rounding (inputs and hidden activations) and FP64
    accumulation. The tolerance covers FP32 accumulation order, the hardware tanh of the
    kernel's GELU (about 2^-11 relative) and an occasional one-ulp difference of a rounded
    activation. 100003 rows are more 128-row tiles than the grid has
    CTAs, so each CTA runs several tiles through the same tensor memory and mbarrier."""
    rng = np.random.default_rng(4)
    mlp = N.Mlp(seed=5)
    w = _weights(rng)
    mlp.set_weights(w)
    for n in (1, 15, 17, 128, 129, 4096 + 5, 100003):
        x = _features(rng, n)
        y = mlp.forward(x)
        ref = M.forward(w, x, emulate_bf16_activations=True)
        scale = np.abs(ref).max() + 1e-3
        assert np.max(np.abs(y - ref)) <= 2e-2 * scale, n
        full = M.forward(w, x)  # and close to the unrounded network
        assert np.max(np.abs(y - full)) <= 8e-2 * (np.abs(full).max() + 1e-3), n


@pytest.mark.gpu
def test_training_fits_a_smooth_map():
    """Adam on the device fits y = tanh(x A) from 20k rows: held-out MSE falls tenfold."""
    rng = np.random.default_rng(6)
    A = rng.normal(size=(24, 3)) * 0.2
    X = _features(rng, 20000) * 0.2
    Y = np.tanh(X @ A).astype(np.float32)
    mlp = N.Mlp(seed=7)
    before = float(np.mean((mlp.forward(X[-2000:]) - Y[-2000:]) ** 2))
    mlp.train(X[:-2000], Y[:-2000], steps=1500, batch=1024, lr=1e-3, seed=1)
    after = float(np.mean((mlp.forward(X[-2000:]) - Y[-2000:]) ** 2))
    assert after < 0.1 * before, (before, after)


def _patch(n=17):
    from spg_gb300 import scenes as S
    return S.spring_cloth(n).objects[0]


@pytest.mark.gpu
def test_zero_network_equals_the_extrapolated_guess():
    """The network only corrects the extrapolated guess: with zero weights the learned mode
    proposes exactly that guess (x_e + l * 0), so its trajectory equals mode 2's bit for bit."""
    obj = _patch()
    kw = dict(dt=1 / 120, iterations=10, gravity=(0, 0, -9.81))
    ext = N.VbdSolver([obj], **kw)
    ext.set_warm_start(None, mode=2)
    warm = N.VbdSolver([obj], **kw)
    mlp = N.Mlp(seed=0, weights=np.zeros(M.N_PARAMS, np.float32))
    warm.set_warm_start(mlp)
    for _ in range(4):
        a = ext.step()
        b = warm.step()
        # The two candidates are the same positions; their FP64 residual sums may differ in
        # the last bits (atomic order), so either may be the one counted.
        assert a.extrapolated_accepted == b.extrapolated_accepted + b.warm_accepted
    assert np.array_equal(ext.state(0)[0], warm.state(0)[0])


@pytest.mark.gpu
def test_worse_learned_guess_is_never_used():
    """A network whose correction is huge makes a guess with a larger residual than both y and
    the extrapolated guess: it is never picked, and the trajectory equals mode 2's bit for bit."""
    obj = _patch()
    kw = dict(dt=1 / 120, iterations=10, gravity=(0, 0, -9.81))
    ext = N.VbdSolver([obj], **kw)
    ext.set_warm_start(None, mode=2)
    warm = N.VbdSolver([obj], **kw)
    w = np.zeros(M.N_PARAMS, np.float32)
    w[M.N_PARAMS - 3:] = 1e4   # b4: a constant correction of 1e4 l (about 7 m) per vertex
    mlp = N.Mlp(seed=0, weights=w)
    warm.set_warm_start(mlp)
    for _ in range(4):
        a = ext.step()
        st = warm.step()
        assert st.warm_accepted == 0
        assert st.extrapolated_accepted == a.extrapolated_accepted
    assert np.array_equal(ext.state(0)[0], warm.state(0)[0])


@pytest.mark.gpu
def test_recorded_features_and_targets():
    """Features recorded at the start of a step equal the definition computed from the host
    states of the three previous steps, and the targets equal (x* - y) / l."""
    obj = _patch()
    h, g = 1 / 120, np.array([0.0, 0.0, -9.81])
    s = N.VbdSolver([obj], dt=h, iterations=10, gravity=tuple(g))
    s.set_warm_start(None, mode=0)
    xs = [s.state(0)[0]]
    for _ in range(3):
        s.step()
        xs.append(s.state(0)[0])
    x_n, v_n = s.state(0)
    st, f, t = s.step_record()
    x_next = s.state(0)[0]
    order = s.vertex_order()
    f = f[np.argsort(order)]
    t = t[np.argsort(order)]
    ell = h * h * 9.81
    d1 = xs[3] - xs[2]
    d2 = xs[2] - xs[1]
    y = x_n + h * (v_n + h * g)
    assert np.allclose(f[:, 0:3], (y - x_n) / ell, atol=2e-3 * max(1, np.abs((y - x_n) / ell).max()))
    assert np.allclose(f[:, 3:6], d1 / ell, atol=2e-3 * max(1, np.abs(d1 / ell).max()))
    assert np.allclose(f[:, 6:9], d2 / ell, atol=2e-3 * max(1, np.abs(d2 / ell).max()))
    # one-ring Laplacian of d1 over the spring edges (every mesh edge carries a spring here)
    springs = next(e for e in obj.energies if e.type == N.SPRING).stencils
    nb = [set() for _ in range(obj.nv)]
    for a, b in springs:
        nb[a].add(b)
        nb[b].add(a)
    lap = np.array([d1[list(nb[i])].mean(0) - d1[i] for i in range(obj.nv)])
    assert np.allclose(f[:, 9:12], lap / ell, atol=2e-3 * max(1, np.abs(lap / ell).max()))
    assert np.allclose(f[:, 15:18], g / 9.81)
    anchored = np.zeros(obj.nv)
    anchored[next(e for e in obj.energies if e.type == N.ANCHOR).stencils[:, 0]] = 1
    assert np.array_equal(f[:, 18], anchored)
    assert np.allclose(f[:, 20], [len(nb[i]) / 8 for i in range(obj.nv)])
    assert np.all(f[:, 23] == 1)
    assert np.allclose(t, (x_next - y) / ell, atol=2e-3 * max(1, np.abs((x_next - y) / ell).max()))
