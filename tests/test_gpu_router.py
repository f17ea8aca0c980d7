"""Medium batches and the learned precision router, through the C ABI.

  * gbs_mbatch_lu_rcond: pivots identical to the CPU oracle, factors within
    1e-12, rcond equal to the oracle's (same algorithm) to 1e-6;
  * gbs_mbatch_ir: items it reports as converged meet backward error 1e-13,
    ill-conditioned items are flagged for FP64;
  * gbs_mbatch_features: equal to a float64 NumPy restatement (FP32 kernel, 2e-3);
  * gbs_mlp_gradients: equal to a float64 NumPy forward/backward (gradient
    check, 2e-3 relative);
  * training lowers the loss and the routed solve beats always-FP64 while every
    result meets the backward-error bound.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from eigen_gb300 import router as R  # noqa: E402


def test_mbatch_lu_rcond_matches_oracle():
    sizes = [1, 2, 5, 17, 33, 64, 100, 129, 200, 257, 300, 512]
    mb = R.MediumBatch(sizes)
    mats = [O.gauss(40 + i, n, n) for i, n in enumerate(sizes)]
    mats[4][:, 7] = 0.0                                       # one exactly singular item
    a = np.concatenate([m.reshape(-1, order="F") for m in mats])
    b = np.concatenate([O.gauss(90 + i, n, 1)[:, 0] for i, n in enumerate(sizes)])
    A = torch.from_numpy(a).cuda()
    X = torch.from_numpy(b).cuda()
    piv = torch.zeros(mb.v_elems, dtype=torch.int32, device="cuda")
    rc = torch.zeros(mb.count, dtype=torch.float64, device="cuda")
    info = torch.zeros(mb.count, dtype=torch.int32, device="cuda")
    mb.lu_rcond(A, piv, X, rc, info)
    torch.cuda.synchronize()
    for i, n in enumerate(sizes):
        f_o, tr_o, _, fz = O.lu(mats[i])
        assert int(info[i]) == fz
        assert np.array_equal(R.MediumBatch.vector(mb, piv, i).cpu().numpy(), tr_o)
        f = mb.matrix(A, i).cpu().numpy()
        assert np.linalg.norm(f - f_o) <= 1e-12 * max(1.0, np.linalg.norm(f_o))
        if fz < 0:
            rc_o = O.lu_rcond(f_o, tr_o, O.l1_norm(mats[i]))
            assert float(rc[i]) == pytest.approx(rc_o, rel=1e-6)
            x = mb.vector(X, i).cpu().numpy()
            assert O.backward_error(mats[i], x.reshape(-1, 1), b[mb.v_off[i]:mb.v_off[i] + n].reshape(-1, 1)) < 1e-14


def test_mbatch_ir_converges_or_flags():
    mb, A, B, logk = R.generate(120, seed=5, nmin=32, nmax=200)
    x, st = R.solve_fp32_ir(mb, A, B)
    st = st.cpu().numpy()
    errs = R.backward_errors(mb, A, x, B)
    ok = st >= 0
    assert ok.any() and (~ok).any()
    assert (errs[ok] <= 1e-13).all()
    assert logk[ok].max() < 10.5 and logk[~ok].min() > 5.0      # easy items converge, hard ones are flagged


def numpy_features(m):
    n = m.shape[0]
    a = m.astype(np.float64)
    rows = np.sqrt((a * a).sum(axis=1))
    fro = np.sqrt((a * a).sum())
    d = np.abs(np.diag(a))
    x = np.array([(1.0 if i % 3 else -1.0) for i in range(n)]) / np.sqrt(n)
    rho = []
    for _ in range(4):
        z = a.T @ (a @ x)
        nn = np.linalg.norm(z)
        rho.append(np.sqrt(nn) / fro)
        x = z / nn
    f = [np.log2(n) / 9, np.linalg.norm(d) / fro, d.min() / d.mean(), d.max() / d.mean(), rows.min() / rows.mean(),
         rows.max() / rows.mean(), np.sqrt(max((rows ** 2).mean() - rows.mean() ** 2, 0)) / rows.mean()]
    f += rho + [10 * np.log(rho[k + 1] / rho[k]) for k in range(3)] + [1.0, 0.0]
    return np.array(f)


def test_features_match_numpy():
    mb, A, _, _ = R.generate(40, seed=6, nmin=32, nmax=300)
    F = R.features(mb, A).cpu().numpy()
    for i in range(mb.count):
        ref = numpy_features(mb.matrix(A, i).cpu().numpy())
        assert np.allclose(F[i], ref, rtol=2e-3, atol=2e-3), (i, F[i], ref)


def numpy_grad(p, X, T, in_dim):
    W = 64
    o = 0
    W1 = p[o:o + in_dim * W].reshape(in_dim, W); o += in_dim * W
    b1 = p[o:o + W]; o += W
    W2 = p[o:o + W * W].reshape(W, W); o += W * W
    b2 = p[o:o + W]; o += W
    W3 = p[o:o + W]; o += W
    b3 = p[o]
    z1 = X @ W1 + b1; h1 = np.maximum(z1, 0)
    z2 = h1 @ W2 + b2; h2 = np.maximum(z2, 0)
    y = h2 @ W3 + b3
    err = y - T
    loss = (err ** 2).mean()
    dy = 2 * err / len(T)
    gW3 = h2.T @ dy; gb3 = dy.sum()
    d2 = np.outer(dy, W3) * (z2 > 0)
    gW2 = h1.T @ d2; gb2 = d2.sum(0)
    d1 = (d2 @ W2.T) * (z1 > 0)
    gW1 = X.T @ d1; gb1 = d1.sum(0)
    return np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]]), loss


def test_mlp_gradients_match_cpu_oracle():
    r = R.Router(seed=3)
    nf = R.feature_count()
    rng = np.random.default_rng(0)
    X = rng.standard_normal((300, nf)).astype(np.float32)
    T = rng.standard_normal(300).astype(np.float32)
    g, loss = r.gradients(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda())
    g_ref, loss_ref = numpy_grad(r.params().astype(np.float64), X.astype(np.float64), T.astype(np.float64), nf)
    assert loss == pytest.approx(loss_ref, rel=1e-5)
    assert np.linalg.norm(g - g_ref) <= 2e-3 * np.linalg.norm(g_ref)


def test_router_trains_and_beats_always_fp64():
    mb, A, B, _ = R.generate(3000, seed=11, nmin=32, nmax=160)
    y = R.labels(mb, A)
    F = R.features(mb, A)
    r = R.Router(seed=1)
    first = r.gradients(F, (y / R.LABEL_SCALE).contiguous())[1]
    final = r.fit(F, y, epochs=40, batch=512, lr=3e-3)
    assert final < 0.25 * first
    pred = r.predict(F)
    err = (pred - y).abs().cpu().numpy()
    assert np.median(err) < 1.0          # within a decade of the method's own estimate
    # routed solve on fresh systems
    mt, At, Bt, _ = R.generate(400, seed=12, nmin=32, nmax=160)
    tier = r.route(r.predict(R.features(mt, At)))
    Xr, stats = R.solve_tiers(mt, At, Bt, tier)
    errs = R.backward_errors(mt, At, Xr, Bt)
    assert (errs <= 1e-13).all()
    assert stats["ir_routed"] > 0 and stats["ir_failed"] <= 0.2 * stats["ir_routed"]
    assert stats["gmres_routed"] > 0 and stats["gmres_failed"] <= 0.5 * stats["gmres_routed"]
    assert stats["fp64_solves"] < mt.count
    # save / load round trip
    import tempfile, os
    path = os.path.join(tempfile.mkdtemp(), "router.json")
    r.save(path)
    r2 = R.Router(seed=99)
    r2.load(path)
    assert np.array_equal(r2.params(), r.params())


def test_mbatch_subset_calls_touch_only_their_items():
    mb, A, B, _ = R.generate(30, seed=21, nmin=32, nmax=100)
    sel = [3, 7, 19, 29]
    X = R.solve_fp64(mb, A, B, items=sel, X=B.clone())
    full = R.solve_fp64(mb, A, B)
    for i in range(mb.count):
        want = mb.vector(full if i in sel else B, i)
        assert torch.equal(mb.vector(X, i), want), i
    F = R.features(mb, A)
    f = torch.full_like(F, 7.0)
    mb.features(A, f, items=R._items(sel))
    for i in range(mb.count):
        assert torch.equal(f[i], F[i]) if i in sel else bool((f[i] == 7.0).all()), i
    x32, st = R.solve_fp32_ir(mb, A, B, items=sel, X=B.clone())
    st = st.cpu().numpy()
    assert set(np.nonzero(st != R.NOT_ATTEMPTED)[0]) == set(sel)
    for i in range(mb.count):
        if st[i] < 0:
            assert torch.equal(mb.vector(x32, i), mb.vector(B, i)), i


def test_mbatch_gmres_ir_extends_the_fp32_tier():
    """Systems FP32 + classic refinement mostly cannot solve (kappa 1e7.5..1e9)
    reach the bound with GMRES-IR on the same FP32 factors."""
    mb, A, B, logk = R.generate(150, seed=31, nmin=32, nmax=300, logk=(7.5, 9.0))
    ws = R.Fp32Work(mb)
    X = B.clone()
    R.solve_fp32_ir(mb, A, B, X=X, ws=ws)
    st_ir = ws.status.cpu().numpy().copy()
    retry = torch.nonzero(ws.status == -1).flatten().to(torch.int32)
    assert retry.numel() > 0.5 * mb.count
    R.solve_fp32_gmres(mb, A, B, items=retry, X=X, ws=ws, factored=True)
    st = ws.status.cpu().numpy()
    inner = ws.inner.cpu().numpy()
    done = st >= 0
    assert done[st_ir == -1].mean() > 0.6, (done[st_ir == -1].mean(), inner[st_ir == -1])
    errs = R.backward_errors(mb, A, X, B)
    assert (errs[done] <= 1e-13).all()
    for i in np.nonzero(~done)[0]:
        assert torch.equal(mb.vector(X, i), mb.vector(B, i)), i


def test_cascade_meets_the_bound_everywhere():
    mb, A, B, _ = R.generate(200, seed=32, nmin=32, nmax=256)
    X, stats = R.solve_cascade(mb, A, B)
    errs = R.backward_errors(mb, A, X, B)
    assert (errs <= 1e-13).all(), (errs.max(), stats)
    assert stats["ir_converged"] > 0 and stats["gmres_converged"] > 0


def test_pretrained_router_routes_fresh_systems():
    """The shipped network (1M rcond labels) on fresh systems of its
    distribution: within half a decade of rcond's estimate, few refinement
    failures, every result within the bound."""
    r = R.Router.pretrained()
    mt, At, Bt, _ = R.generate(300, seed=41, nmin=32, nmax=512)
    err = (r.predict(R.features(mt, At)) - R.labels(mt, At)).abs().cpu().numpy()
    assert np.median(err) < 0.6
    X, stats = R.route_and_solve(r, mt, At, Bt)
    assert (R.backward_errors(mt, At, X, Bt) <= 1e-13).all()
    routed = stats["ir_routed"] + stats["gmres_routed"]
    assert routed > 0.3 * mt.count
    assert stats["ir_failed"] + stats["gmres_failed"] <= 0.05 * routed


def test_router_gain_over_the_cascade():
    """What the shipped network gains over the same solver chain without it,
    on the same seeded systems (n 32..512, log10 kappa uniform in 1..12): the
    try-lowest cascade (every item FP32 + refinement, GMRES-IR on the items it
    leaves, FP64 on the rest) against route-and-solve.  The router must make
    fewer failed refinement attempts and fewer factorizations, and take less
    wall time; both must meet the backward-error bound on every item."""
    from tests.conftest import record_note
    mb, A, B, logk = R.generate(1500, seed=31)
    router = R.Router.pretrained()
    for _ in range(2):                                   # warm-up: kernels, workspaces, autotune entries
        R.solve_cascade(mb, A, B)
        R.route_and_solve(router, mb, A, B)
    tc, tr = [], []
    for _ in range(3):
        (Xc, sc), t = R.timed(lambda: R.solve_cascade(mb, A, B))
        tc.append(t)
        (Xr, sr), t = R.timed(lambda: R.route_and_solve(router, mb, A, B))
        tr.append(t)
    tc, tr = float(np.median(tc)), float(np.median(tr))
    n = mb.count
    casc_failed = (n - sc["ir_converged"]) + (sc["gmres_attempts"] - sc["gmres_converged"])
    casc_factor = n + sc["fp64_solves"]                  # one FP32 LU per item (GMRES reuses it) + FP64 LUs
    rout_failed = sr["ir_failed"] + sr["gmres_failed"]
    rout_factor = sr["ir_routed"] + sr["gmres_routed"] + sr["fp64_solves"]
    record_note("router vs cascade, 1500 systems",
                f"failed refinement attempts {rout_failed} vs {casc_failed}; factorizations {rout_factor} vs "
                f"{casc_factor}; wall {tr * 1e3:.1f} ms vs {tc * 1e3:.1f} ms ({tc / tr:.2f}x)")
    for X in (Xc, Xr):
        errs = R.backward_errors(mb, A, X, B)
        assert (errs <= 1e-13).all(), float(errs.max())
    assert rout_failed < casc_failed
    assert rout_factor < casc_factor
    assert tr < tc, (tr, tc)
