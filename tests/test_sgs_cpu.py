"""The learned-closure oracle on the CPU: its MLP gradient against central
finite differences of its own loss, its features against an independent
numpy restatement, and the box filter / subgrid-stress target on fields
with known answers."""
from __future__ import annotations

import ctypes

import numpy as np

from oracle_bindings import oracle, ptr

NIN, NH = 16, 64
NPARAM = NH * NIN + NH * NH + NH + NH + 1


def _params(seed=3, scale=0.3):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(NPARAM) * scale).astype(np.float32)


def _samples(n, seed=4):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, NIN)).astype(np.float32)
    X[:, 15] = 1
    T = (rng.random(n) * 3e-4).astype(np.float32)
    return X, T


def _loss(o, P, X, T):
    g = np.zeros(NPARAM)
    L = ctypes.c_double()
    o.orc_mlp_grad(ptr(P), ptr(X), ptr(T), len(T), ptr(g), ctypes.byref(L))
    return L.value, g


def test_oracle_gradient_matches_finite_differences():
    o = oracle()
    assert o.orc_mlp_nparam() == NPARAM
    P = _params()
    X, T = _samples(24)
    L0, g = _loss(o, P, X, T)
    rng = np.random.default_rng(9)
    # a spread of parameters from every block: W1, W1 bias column, W2, b2, w3, b3
    picks = list(rng.choice(NH * NIN, 8, replace=False)) + [15, 16 * 7 + 15]
    picks += list(NH * NIN + rng.choice(NH * NH, 8, replace=False))
    picks += [NH * NIN + NH * NH + 5, NH * NIN + NH * NH + NH + 9, NPARAM - 1]
    for p in picks:
        # a small step: the ReLU loss is smooth only between kinks (a sample's
        # pre-activation crossing zero), and the FP64 loss resolves 1e-5 well
        h = 1e-5 * max(1.0, abs(float(P[p])))
        Pp, Pm = P.copy(), P.copy()
        Pp[p] += h
        Pm[p] -= h
        h = (float(Pp[p]) - float(Pm[p])) / 2  # the step the float32 params really took
        fd = (_loss(o, Pp, X, T)[0] - _loss(o, Pm, X, T)[0]) / (2 * h)
        assert abs(fd - g[p]) <= 2e-4 * max(1.0, abs(g[p])), (p, fd, g[p])
    assert L0 > 0


def _forward_np(P, X):
    """the network restated in numpy: W1 (column 15 the bias against x15 =
    1), ReLU, hidden unit 63 the constant 1 whatever row 63 of W1 holds, W2
    + b2, ReLU, w3 + b3, softplus, times 1e-4"""
    W1 = P[: NH * NIN].reshape(NH, NIN).astype(np.float64)
    o = NH * NIN
    W2 = P[o: o + NH * NH].reshape(NH, NH).astype(np.float64)
    o += NH * NH
    b2, w3, b3 = P[o: o + NH].astype(np.float64), P[o + NH: o + 2 * NH].astype(np.float64), float(P[-1])
    h1 = np.maximum(X.astype(np.float64) @ W1.T, 0)
    h1[:, NH - 1] = 1
    h2 = np.maximum(h1 @ W2.T + b2, 0)
    y = h2 @ w3 + b3
    return 1e-4 * np.logaddexp(0, y)


def test_oracle_forward_matches_numpy():
    """the oracle's MLP against the numpy restatement above, on parameters
    whose row 63 of W1 is not e15 (the constant unit ignores it) and on
    samples that drive units to both sides of the ReLU kink"""
    o = oracle()
    P = _params(seed=11, scale=0.4)
    X, _ = _samples(257, seed=12)
    got = np.zeros(len(X))
    o.orc_mlp_forward(ptr(P), ptr(X), len(X), ptr(got))
    want = _forward_np(P, X)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-18)
    # the constant unit: changing row 63 of W1 changes nothing
    P2 = P.copy()
    P2[(NH - 1) * NIN: NH * NIN] = 5.0
    got2 = np.zeros(len(X))
    o.orc_mlp_forward(ptr(P2), ptr(X), len(X), ptr(got2))
    np.testing.assert_array_equal(got, got2)
    # and both ReLU branches are live in layer 1
    z1 = X.astype(np.float64) @ P[: NH * NIN].reshape(NH, NIN).astype(np.float64).T
    assert (z1 > 0).mean() > 0.2 and (z1 < 0).mean() > 0.2


def _features_np(p, tau0):
    m = np.array([[p[0], p[3], p[4]], [p[3], p[1], p[5]], [p[4], p[5], p[2]]])
    pp = float((m * m).sum())
    x = np.zeros(16)
    x[12] = np.sqrt(2 * pp) / 0.01
    x[13] = np.trace(m @ m @ m) / pp ** 1.5 if pp > 1e-30 else 0.0
    x[14] = (tau0 - 0.5) * 100
    x[15] = 1
    return x


def test_oracle_features():
    o = oracle()
    rng = np.random.default_rng(1)
    for _ in range(20):
        p = rng.standard_normal(6) * 1e-3
        tau0 = 0.5 + rng.random() * 0.1
        x = np.zeros(16)
        o.orc_sgs_features(ptr(p), ctypes.c_double(tau0), ptr(x))
        np.testing.assert_allclose(x, _features_np(p, tau0), rtol=1e-12, atol=1e-12)
    x = np.zeros(16)
    o.orc_sgs_features(ptr(np.zeros(6)), ctypes.c_double(0.55), ptr(x))
    assert x[13] == 0 and x[15] == 1


def test_oracle_box_filter_and_target():
    o = oracle()
    fx = fy = fz = 16
    z, y, x = np.meshgrid(np.arange(fz), np.arange(fy), np.arange(fx), indexing="ij")
    # a field constant over each 2x2x2 block has no subgrid stress
    blk = np.sin(2 * np.pi * (x // 2) / 8) * 0.01
    u = np.stack([blk, 0 * blk, 0 * blk]).astype(np.float32)
    ub = np.zeros((3, 8, 8, 8))
    uu = np.zeros((6, 8, 8, 8))
    o.orc_box_filter(ptr(u), fx, fy, fz, ptr(ub), ptr(uu))
    np.testing.assert_allclose(ub[0], blk[::2, ::2, ::2], atol=1e-9)
    X = np.zeros((512, 16), np.float32)
    T = np.zeros(512, np.float32)
    o.orc_sgs_targets(ptr(ub), ptr(uu), 8, 8, 8, ctypes.c_double(0.52), ptr(X), ptr(T))
    assert np.abs(T).max() < 1e-12
    assert np.all(X[:, 15] == 1)
    # a random field that varies inside the blocks: non-negative eddy
    # viscosity, positive where the subgrid stress drains the resolved strain
    u2 = (np.random.default_rng(5).standard_normal((3, fz, fy, fx)) * 0.01).astype(np.float32)
    o.orc_box_filter(ptr(u2), fx, fy, fz, ptr(ub), ptr(uu))
    o.orc_sgs_targets(ptr(ub), ptr(uu), 8, 8, 8, ctypes.c_double(0.52), ptr(X), ptr(T))
    assert T.min() >= 0 and T.max() > 0


def test_host_samples_match_the_oracle_on_a_periodic_field(orc):
    """the host sample extraction used for channel runs (samples_from_velocity,
    features_np) reproduces the oracle's box filter, least-squares targets
    and features on a periodic field (all fluid, no margin)"""
    from lbm_multigpu_gb300.sgs_pipeline import samples_from_velocity

    rng = np.random.default_rng(5)
    fz, fy, fx = 12, 16, 20
    u = (0.03 * rng.standard_normal((3, fz, fy, fx))).astype(np.float32)
    ub = np.zeros(3 * (fx // 2) * (fy // 2) * (fz // 2))
    uu = np.zeros(6 * (fx // 2) * (fy // 2) * (fz // 2))
    n = (fx // 2) * (fy // 2) * (fz // 2)
    Xo, To = np.zeros((n, 16), np.float32), np.zeros(n, np.float32)
    orc.orc_box_filter(ptr(u), fx, fy, fz, ptr(ub), ptr(uu))
    orc.orc_sgs_targets(ptr(ub), ptr(uu), fx // 2, fy // 2, fz // 2, ctypes.c_double(0.505), ptr(Xo), ptr(To))
    X, T = samples_from_velocity(u, np.ones((fz, fy, fx), bool), 0.505, margin=0)
    assert X.shape == (n, 16) and (To > 0).mean() > 0.2
    np.testing.assert_allclose(T, To, rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(X, Xo, rtol=1e-4, atol=1e-5)


def test_host_samples_stay_clear_of_solids():
    """cells within the margin of a non-fluid node or a non-periodic edge
    give no sample"""
    from lbm_multigpu_gb300.sgs_pipeline import samples_from_velocity

    rng = np.random.default_rng(6)
    u = (0.02 * rng.standard_normal((3, 8, 24, 24))).astype(np.float32)
    fluid = np.ones((8, 24, 24), bool)
    X, _ = samples_from_velocity(u, fluid, 0.505, margin=2)
    assert len(X) == 4 * 8 * 8           # 12 x 12 coarse cells less 2 on each side in x and y
    fluid[:, 10:12, 10:12] = False       # one coarse column solid
    X2, _ = samples_from_velocity(u, fluid, 0.505, margin=2)
    assert len(X2) == 4 * (64 - 25)      # the 5 x 5 cells around it drop out (all inside the interior)


def test_regularised_targets_vanish_where_the_strain_is_weak():
    """reg > 0: nu = max(0, -<tau:S>) / (2 (<S:S> + reg mean<S:S>)) keeps the
    plain fit where the strain is strong and goes to zero where it is weak"""
    from lbm_multigpu_gb300.sgs_pipeline import samples_from_velocity

    rng = np.random.default_rng(8)
    u = (0.03 * rng.standard_normal((3, 12, 16, 20))).astype(np.float32)
    u[:, :, :, :10] *= 1e-3                  # a quiet half: weak strain, noise-level stress
    fl = np.ones(u.shape[1:], bool)
    X0, T0 = samples_from_velocity(u, fl, 0.52, margin=0)
    X1, T1 = samples_from_velocity(u, fl, 0.52, margin=0, reg=0.25)
    assert X0.shape == X1.shape      # the features carry each fit's own nu: p = (tau0 + 3 nu) S
    assert (T1 <= T0 + 1e-12).all()
    s = X0[:, 12]
    strong, weak = s > np.percentile(s, 75), s < np.percentile(s, 25)
    pos = strong & (T0 > 0)
    assert pos.sum() > 10 and np.median(T1[pos] / T0[pos]) > 0.5
    assert T1[weak].sum() < 1e-2 * T0[weak].sum()


def test_coefficient_targets_invert_the_strain_gain():
    """the collision's eddy viscosity is o x12 / tau0: the coefficient
    targets times that gain give back the eddy-viscosity targets (below the
    cap), zero where x12 is zero, and the oracle collision applies the same
    gain"""
    from lbm_multigpu_gb300.sgs_pipeline import coefficient_targets

    X, T = _samples(256)
    X[:, 12] = np.abs(X[:, 12])
    X[:5, 12] = 0
    X[:, 14] = 2.0
    o = coefficient_targets(X, T)
    g = X[:, 12] / (X[:, 14] / 100 + 0.5)
    ok = (g > 0) & (T / np.where(g > 0, g, 1) < 5e-3)
    np.testing.assert_allclose(o[ok] * g[ok], T[ok], rtol=1e-6)
    assert (o[:5] == 0).all() and (o <= 5e-3).all()
    # oracle: nu_out = 1e-4 softplus(y) x12 / tau0 with x from the node's stress
    rng = np.random.default_rng(9)
    from oracle_bindings import W as WQ

    f = np.tile(WQ, (4, 1)) * (1 + 0.01 * rng.standard_normal((4, 19)))
    P = _params(5, 0.2)
    nu = np.zeros(4)
    orc = oracle()
    g2 = f.copy()
    orc.orc_collide_mlp(ptr(P), ctypes.c_double(0.52), ptr(g2), 4, ptr(nu))
    for i in range(4):
        rho, pi = ctypes.c_double(), np.zeros(6)
        orc.orc_pi_neq(ptr(f[i]), ctypes.byref(rho), ptr(pi))
        x = np.zeros(16)
        orc.orc_sgs_features(ptr(pi * (-1.5 / rho.value)), ctypes.c_double(0.52), ptr(x))
        y = np.zeros(1)
        orc.orc_mlp_forward(ptr(P), ptr(x.astype(np.float32)), 1, ptr(y))
        np.testing.assert_allclose(nu[i], y[0] * x[12] / 0.52, rtol=1e-6)


def test_oracle_refresh_schedule():
    """orc_params.mlp_every: on a refresh step (t % k == 0) the oracle's
    step equals the every-step closure's and stores each node's nu_t
    (non-negative, finite); on the steps between it relaxes with the stored
    values, so the two schedules part after the first step"""
    from oracle_bindings import OracleRun

    rng = np.random.default_rng(12)
    nx, ny, nz = 12, 8, 4
    mask = np.zeros((nz, ny, nx), np.uint8)
    mask[:, 0, :] = mask[:, -1, :] = 1
    P = _params(7, 0.2)
    P[-1] = 10.0
    runs = [OracleRun(nx, ny, nz, mask, 1 / 0.52, model=0, les=0, init_kind=0, init_u=0.0, mlp=P, mlp_every=k)
            for k in (1, 4)]
    f0 = runs[0].fa * (1 + 0.01 * rng.standard_normal(runs[0].fa.shape)).astype(np.float32)  # a stressed state
    for o in runs:
        o.fa[:] = f0
        o.fb[:] = f0
    for o in runs:
        o.step(1)
    np.testing.assert_array_equal(runs[0].fa, runs[1].fa)
    nu = runs[1]._nu.reshape(nz, ny, nx)[:, 1:-1, :]
    assert np.isfinite(nu).all() and (nu >= 0).all() and nu.max() > 0
    for o in runs:
        o.step(2)
    assert np.abs(runs[0].fa - runs[1].fa).max() > 0


def _bf16(a):
    """round FP32 to bf16 (nearest even) and back to FP32"""
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32)


def _core(blob, rows, k, sbo):
    """a bf16 matrix [rows][k] read back from the K-major core-matrix layout"""
    out = np.zeros((rows, k), np.float32)
    for r in range(rows):
        for c in range(k):
            off = (r // 8) * sbo + (c // 8) * 128 + (r % 8) * 16 + (c % 8) * 2
            out[r, c] = (np.frombuffer(blob[off: off + 2], "<u2").astype(np.uint32) << 16).view(np.float32)[0]
    return out


def test_weight_blob_folds_the_biases(product):
    """the tensor-core weight blob from a parameter vector: W1 with the
    constant unit's row e15, W2 with b2 folded into column 63, the output
    layer as row 0 of a 16-row W3, b3 in FP32 -- all bf16 in the core-matrix
    layout the MMA descriptors read"""
    lib = product.library()
    P = _params(seed=5, scale=0.5)
    nb = lib.lbm_mlp_blob_bytes()
    blob = np.zeros(nb, np.uint8)
    assert lib.lbm_mlp_make_blob(ptr(P), ptr(blob)) == 0
    raw = blob.tobytes()
    o = NH * NIN
    W1, W2 = P[:o].reshape(NH, NIN), P[o: o + NH * NH].reshape(NH, NH)
    b2, w3, b3 = P[o + NH * NH: o + NH * NH + NH], P[o + NH * NH + NH: o + NH * NH + 2 * NH], P[-1]
    want1 = W1.copy()
    want1[NH - 1] = 0
    want1[NH - 1, NIN - 1] = 1
    np.testing.assert_array_equal(_core(raw[: NH * NIN * 2], NH, NIN, 256), _bf16(want1))
    w2_off = NH * NIN * 2
    want2 = W2.copy()
    want2[:, NH - 1] = W2[:, NH - 1] + b2
    np.testing.assert_array_equal(_core(raw[w2_off: w2_off + NH * NH * 2], NH, NH, 1024), _bf16(want2))
    w3_off = w2_off + NH * NH * 2
    got3 = _core(raw[w3_off: w3_off + 16 * NH * 2], 16, NH, 1024)
    np.testing.assert_array_equal(got3[0], _bf16(w3))
    assert not got3[1:].any()
    b3_off = w3_off + 16 * NH * 2
    assert np.frombuffer(raw[b3_off: b3_off + 4], "<f4")[0] == b3
    assert nb == b3_off + 16 and not blob[b3_off + 4:].any()


def test_bf16_inference_error_is_within_the_gpu_tolerance(product):
    """the tensor-core inference's rounding, emulated: bf16 features, the
    blob's bf16 weights, FP32 accumulation, ReLU then bf16 for the first
    hidden layer, the output layer in FP32 from the second's accumulators,
    b3 in FP32.  Its distance to the FP64 oracle forward on the GPU test's
    inputs stays inside that test's 0.6 % (rounding alone accounts for it,
    and is not zero: the tolerance is not slack), and the oracle's own
    emulation of the same rounding (orc_mlp_set_bf16) agrees with it"""
    lib = product.library()
    rng = np.random.default_rng(8)
    P = np.zeros(NPARAM, np.float32)
    assert lib.lbm_mlp_init_params(13, ptr(P)) == 0
    P[NH * NIN + NH * NH: NH * NIN + NH * NH + NH] = 0.1
    X = (rng.standard_normal((3000, NIN)) * 0.7).astype(np.float32)
    X[:, 15] = 1
    blob = np.zeros(lib.lbm_mlp_blob_bytes(), np.uint8)
    assert lib.lbm_mlp_make_blob(ptr(P), ptr(blob)) == 0
    raw = blob.tobytes()
    w2_off = NH * NIN * 2
    w3_off = w2_off + NH * NH * 2
    W1 = _core(raw[:w2_off], NH, NIN, 256).astype(np.float64)
    W2 = _core(raw[w2_off:w3_off], NH, NH, 1024).astype(np.float64)
    w3 = _core(raw[w3_off: w3_off + 16 * NH * 2], 16, NH, 1024)[0].astype(np.float64)
    b3 = float(np.frombuffer(raw[w3_off + 16 * NH * 2: w3_off + 16 * NH * 2 + 4], "<f4")[0])
    h1 = _bf16(np.maximum((_bf16(X).astype(np.float64) @ W1.T).astype(np.float32), 0)).astype(np.float64)
    h2 = np.maximum((h1 @ W2.T).astype(np.float32), 0).astype(np.float64)
    y = (h2 @ w3).astype(np.float32).astype(np.float64) + b3
    emulated = 1e-4 * np.logaddexp(0, y)
    want = np.zeros(len(X))
    oracle().orc_mlp_forward(ptr(P), ptr(X), len(X), ptr(want))
    err = np.linalg.norm(emulated - want) / np.linalg.norm(want)
    assert 1e-5 < err < 6e-3, err
    emu = np.zeros(len(X))
    oracle().orc_mlp_set_bf16(1)
    try:
        oracle().orc_mlp_forward(ptr(P), ptr(X), len(X), ptr(emu))
    finally:
        oracle().orc_mlp_set_bf16(0)
    assert np.linalg.norm(emu - emulated) / np.linalg.norm(want) < 1e-5
