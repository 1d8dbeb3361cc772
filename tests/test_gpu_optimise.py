"""GPU finite-difference consumers: the Hessian and gradient batches
against the same points evaluated one request at a time, against the
oracle's evaluations, and the errors() pipeline on top."""
import numpy as np
import pytest

from conftest import load_case

pytestmark = pytest.mark.gpu


def _setup(ctx, name):
    import milkywayathome_client_gb300 as mw
    pf, sf, g = load_case(name)
    ap = mw.AstronomyParameters.read(pf)
    ctx.set_problem(ap)
    ctx.set_stars(mw.StarPoints.read(sf))
    return pf, sf, g, ap


def _points(theta, step):
    """The library's point order: centre, +/-h_i, then (++,+-,-+,--) per i<j."""
    P = len(theta)
    pts = [np.array(theta, float)]
    for i in range(P):
        for s in (+1, -1):
            p = np.array(theta, float)
            p[i] += s * step[i]
            pts.append(p)
    for i in range(P):
        for j in range(i + 1, P):
            for si, sj in ((1, 1), (1, -1), (-1, 1), (-1, -1)):
                p = np.array(theta, float)
                p[i] += si * step[i]
                p[j] += sj * step[j]
                pts.append(p)
    return pts


def _assemble(f, step):
    P = len(step)
    fc = f[0]
    g = np.array([(f[1 + 2 * i] - f[2 + 2 * i]) / (2.0 * step[i]) for i in range(P)])
    H = np.zeros((P, P))
    for i in range(P):
        H[i, i] = ((f[1 + 2 * i] - fc) + (f[2 + 2 * i] - fc)) / (step[i] * step[i])
    k = 1 + 2 * P
    for i in range(P):
        for j in range(i + 1, P):
            H[i, j] = H[j, i] = ((f[k] - f[k + 1]) - (f[k + 2] - f[k + 3])) / (4.0 * step[i] * step[j])
            k += 4
    return fc, g, H


@pytest.mark.parametrize("precision", [0, 1])
def test_hessian_equals_pointwise_assembly(gpu_ctx, precision):
    _, _, g, ap = _setup(gpu_ctx, "three_streams")
    theta = g["theta"]
    step = ap.step()
    f0, grad, H = gpu_ctx.hessian(0, theta, step, precision)
    res = gpu_ctx.evaluate_requests([(0, p) for p in _points(theta, step)], precision)
    fc, g2, H2 = _assemble([r.likelihood for r in res], step)
    assert f0 == fc
    assert np.array_equal(grad, g2)
    assert np.array_equal(H, H2)
    assert np.array_equal(H, H.T)
    f0b, grad_b = gpu_ctx.gradient(0, theta, step, precision)
    assert f0b == f0 and np.array_equal(grad_b, grad)


def test_hessian_matches_oracle(gpu_ctx, oracle_built):
    pf, sf, g, ap = _setup(gpu_ctx, "basic_1stream")
    theta = g["theta"]
    step = ap.step()
    f0, grad, H = gpu_ctx.hessian(0, theta, step, 0)
    o = oracle_built.Oracle(pf, sf)
    f = [o.evaluate(p)["likelihood"] for p in _points(theta, step)]
    fc, g2, H2 = _assemble(f, step)
    assert abs(f0 - fc) <= 1e-12
    # |delta f| <= 1e-12 per point, divided by the step products
    hh = np.outer(step, step)
    assert np.all(np.abs(H - H2) <= 4e-12 / hh + 1e-9 * np.abs(H2))
    assert np.all(np.abs(grad - g2) <= 1e-12 / step + 1e-9 * np.abs(g2))


def test_mixed_hessian_close_to_plain(gpu_ctx):
    _, _, g, ap = _setup(gpu_ctx, "three_streams")
    step = ap.step()
    fp, gp, Hp = gpu_ctx.hessian(0, g["theta"], step, 0)
    fm, gm, Hm = gpu_ctx.hessian(0, g["theta"], step, 1)
    # per evaluation the compensated form is within EPS of the plain one on
    # this case (its contract is 1e-7); a central-difference entry amplifies
    # that by at most 4 / (h_i h_j), a gradient entry by 1 / h_i
    EPS = 1e-8
    assert abs(fm - fp) <= EPS
    hh = np.outer(step, step)
    assert np.all(np.abs(Hm - Hp) <= 4 * EPS / hh)
    assert np.all(np.abs(gm - gp) <= EPS / step)


def test_errors_pipeline(gpu_ctx, tmp_path):
    import milkywayathome_client_gb300 as mw
    _, _, g, ap = _setup(gpu_ctx, "basic_1stream")
    step = ap.step()
    _, _, H = gpu_ctx.hessian(0, g["theta"], step, 0)
    n_stars = 600
    sigma, sd = mw.errors_from_hessian(H, n_stars)
    np.testing.assert_allclose(sigma @ H * n_stars, np.eye(H.shape[0]), atol=1e-8)
    assert np.all(np.isfinite(sd))
    mw.write_errors(str(tmp_path / "errors.txt"), H, sigma, sd)


def test_hessian_rejects_bad_steps(gpu_ctx):
    import milkywayathome_client_gb300 as mw
    _, _, g, ap = _setup(gpu_ctx, "basic_1stream")
    step = ap.step()
    step[0] = 0.0
    with pytest.raises(mw.MwsepError):
        gpu_ctx.hessian(0, g["theta"], step, 0)
