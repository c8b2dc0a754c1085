"""Tally derivatives: the likelihood-ratio backward kernel against central
finite differences with common random numbers and against the deterministic
(S_N) derivative of the homogeneous one-group slab."""
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mc():
    import build as B
    B.build()
    import mcgpu
    return mcgpu


def _layered(d, tot, c):
    import mcgpu.workloads as W
    W.mg_layered_slab(d, samples=1000, n_regions=len(tot), tot=tot, c=c)


def test_forward_matches_replay(mc):
    """mc_forward at the problem's own parameters is the FP64 replay run."""
    with tempfile.TemporaryDirectory() as d:
        rng = np.random.default_rng(5)
        _layered(d, rng.uniform(0.2, 0.5, 16), rng.uniform(0.3, 0.95, 16))
        p = mc.Problem(d)
        par = p.lr_params()
        assert par.size == 32
        m, s = p.forward(par, 20000, seed=11)
        p.run(n=20000, seed=11, mode="replay")
        m2, s2, _, _ = p.all_tallies()
        p.close()
    assert np.array_equal(m, m2) and np.allclose(s, s2, rtol=1e-12)


def _fd(p, par, k, rel, batches, nb):
    h = rel * par[k]
    out = np.zeros(batches)
    for b in range(batches):
        up, dn = par.copy(), par.copy()
        up[k] += h
        dn[k] -= h
        tu, _ = p.forward(up, nb, seed=1000 + b)
        td, _ = p.forward(dn, nb, seed=1000 + b)
        out[b] = (tu[0] - td[0]) / (2 * h)
    return out.mean(), out.std(ddof=1) / np.sqrt(batches)


@pytest.mark.parametrize("rel,frac2,zmax", [(1e-3, 0.8, 5.0), (1e-2, 0.85, 4.5)])
def test_backward_matches_finite_differences(mc, rel, frac2, zmax):
    """32 gradients (Sigma_s, Sigma_a of 16 regions) vs central differences
    with common random numbers; the FD noise comes from 24 independent
    batches.  With common random numbers a perturbation flips a few
    collide-or-cross decisions and those histories then diverge, so the FD
    estimate is a sum of rare large jumps and its noise falls only as
    1/sqrt(step): the 1e-3 step (as specified) is checked at a looser bar
    than the 1e-2 step.  A fair 2-sigma test misses ~5 % of the parameters."""
    with tempfile.TemporaryDirectory() as d:
        rng = np.random.default_rng(7)
        _layered(d, rng.uniform(0.125, 0.5, 16), rng.uniform(0.3, 0.95, 16))
        p = mc.Problem(d)
        par = p.lr_params()
        g, gs = p.backward(par, 800_000, seed=3)
        g, gs = g[0], gs[0]
        fd = np.array([_fd(p, par, k, rel, 24, 50_000) for k in range(par.size)])
        p.close()
    z = np.abs(g - fd[:, 0]) / np.sqrt(gs ** 2 + fd[:, 1] ** 2)
    table = "\n".join(f"k={k:2d} lr={g[k]: .5e}+-{gs[k]:.1e} fd={fd[k, 0]: .5e}+-{fd[k, 1]:.1e} z={z[k]:.2f}"
                       for k in range(par.size))
    assert np.mean(z <= 2.0) >= frac2 and np.all(z <= zmax), table


def test_backward_on_the_differentiation_configuration(mc):
    """The differentiation workload exactly as configured: 16 x 1 cm layers
    with Sigma_t ~ U[0.5, 2] and c ~ U[0.3, 0.95] (about 22 mean free paths),
    10^7 histories.  Its transmitted current is ~5e-9 (S_N): at 10^7
    histories it is scored a handful of times (R ~ 45 %), so resolved
    detector tallies sit beside it: the reflected current and the current
    through every interface.  The backward kernel's gradients of all 19
    bins with respect to the 32 parameters are compared with central finite
    differences (relative step 1e-3, common random numbers, 40 independent
    batches of 2.5e5 histories).

    The bar is set on the bins whose tally the run resolves (R <= 1 % at
    10^7 histories: the reflected current and the interfaces down to 6 cm):
    there at least 90 % of the gradients lie within 2 sigma and all within
    4.5 sigma, and so do the reflected current's 32.  A gradient neither
    estimator can see (a layer too deep to reach and come back from) is
    exactly zero in both.  Deeper bins (R from 1 % to 50 %) are scored by
    a few rare histories; there the per-history scores are heavy-tailed and
    the standard errors of both estimators are themselves unreliable, so
    their agreement is printed, not asserted."""
    import mcgpu.workloads as W
    n_lr, batches, n_fd, rel = 10_000_000, 40, 250_000, 1e-3
    with tempfile.TemporaryDirectory() as d:
        W.mg_layered_slab(d, samples=1000, detectors=True)
        p = mc.Problem(d)
        names = list(p.names)
        par = p.lr_params()
        assert par.size == 32
        g, gs = p.backward(par, n_lr, seed=3)
        m0, s0 = p.forward(par, n_lr, seed=3)
        fd = np.zeros((batches, g.shape[0], par.size))
        for k in range(par.size):
            h = rel * par[k]
            for b in range(batches):
                up, dn = par.copy(), par.copy()
                up[k] += h
                dn[k] -= h
                tu, _ = p.forward(up, n_fd, seed=1000 + b)
                td, _ = p.forward(dn, n_fd, seed=1000 + b)
                fd[b, :, k] = (tu - td) / (2 * h)
        p.close()
    assert names == ["transmitted", "reflected", "interfaces"] and g.shape == (19, 32)
    fm = fd.mean(axis=0)
    fsd = fd.std(axis=0, ddof=1) / np.sqrt(batches)
    var = gs ** 2 + fsd ** 2
    seen = var > 0
    assert np.all(g[~seen] == 0) and np.all(fm[~seen] == 0), "a gradient is nonzero with zero variance"
    z = np.where(seen, np.abs(g - fm) / np.sqrt(np.where(seen, var, 1.0)), 0.0)
    R = np.where(m0 != 0, s0 / np.where(m0 != 0, np.abs(m0), 1.0), np.inf)
    resolved = (R <= 0.01)[:, None] & seen
    for b in range(19):
        zz = z[b][seen[b]]
        print(f"LR config 5 bin {b:2d} R={R[b]:.2e}: {zz.size} gradients seen, "
              f"{np.mean(zz <= 2.0) if zz.size else 1.0:.2f} within 2 sigma, max z {zz.max() if zz.size else 0:.2f}")
    refl = z[1]
    table = "\n".join(f"reflected k={k:2d} lr={g[1, k]: .4e}+-{gs[1, k]:.1e} fd={fm[1, k]: .4e}+-{fsd[1, k]:.1e} "
                       f"z={refl[k]:.2f}" for k in range(32))
    assert R[1] <= 0.01 and resolved.sum() >= 100
    frac = float(np.mean(z[resolved] <= 2.0))
    print(f"LR config 5: {int(resolved.sum())} gradients of resolved bins, {frac:.3f} within 2 sigma, "
          f"max z {z[resolved].max():.2f}")
    assert frac >= 0.9 and z[resolved].max() <= 4.5, table
    assert np.mean(refl <= 2.0) >= 0.9, table


def test_backward_matches_deterministic_derivative(mc):
    """Homogeneous 1-group slab (16 x 0.25 cm, Sigma_t = 1, c = 0.5): LR
    derivatives of the transmitted current vs central differences of the
    S_N solution, for a few regions."""
    from analytic import solve_slab
    R, w = 16, 0.25
    tot, c = np.full(R, 1.0), np.full(R, 0.5)
    with tempfile.TemporaryDirectory() as d:
        import mcgpu.workloads as W
        W.mg_layered_slab(d, samples=1000, n_regions=R, tot=tot, c=c)
        # the writer makes 1 cm regions; rewrite the plane positions for 0.25 cm
        import re
        txt = open(d + "/input.xml").read()
        txt = re.sub(r'<plane_x name="p(\d+)" x="[^"]*"/>',
                     lambda m_: f'<plane_x name="p{m_.group(1)}" x="{int(m_.group(1)) * w!r}"/>', txt)
        open(d + "/input.xml", "w").write(txt)
        p = mc.Problem(d)
        par = p.lr_params()
        g, gs = p.backward(par, 2_000_000, seed=5)
        m, s = p.forward(par, 2_000_000, seed=5)
        p.close()
    ss, sa = par[0::2], par[1::2]
    base = solve_slab([w] * R, ss + sa, ss, n_mu=48, dx_max=0.0125)
    assert abs(m[0] - base["transmission"]) <= 4 * s[0]
    for r in (0, 5, 10, 15):
        for k, which in ((2 * r, "s"), (2 * r + 1, "a")):
            h = 1e-4
            up_s, up_a = ss.copy(), sa.copy()
            dn_s, dn_a = ss.copy(), sa.copy()
            if which == "s":
                up_s[r] += h
                dn_s[r] -= h
            else:
                up_a[r] += h
                dn_a[r] -= h
            tu = solve_slab([w] * R, up_s + up_a, up_s, n_mu=48, dx_max=0.0125)["transmission"]
            td = solve_slab([w] * R, dn_s + dn_a, dn_s, n_mu=48, dx_max=0.0125)["transmission"]
            exact = (tu - td) / (2 * h)
            assert abs(g[0, k] - exact) <= 4 * gs[0, k] + 1e-3 * abs(exact), (r, which, g[0, k], exact, gs[0, k])


def test_density_derivatives(mc):
    """rho d(T)/d(rho) per region from the same backward run: equal to
    Sigma_s dT/dSigma_s + Sigma_a dT/dSigma_a, with its own per-history
    standard error, and equal to the S_N derivative for a density scaling
    of one region of the homogeneous slab."""
    from analytic import solve_slab
    R, w = 16, 0.25
    tot, c = np.full(R, 1.0), np.full(R, 0.5)
    with tempfile.TemporaryDirectory() as d:
        import mcgpu.workloads as W
        W.mg_layered_slab(d, samples=1000, n_regions=R, tot=tot, c=c)
        import re
        txt = open(d + "/input.xml").read()
        txt = re.sub(r'<plane_x name="p(\d+)" x="[^"]*"/>',
                     lambda m_: f'<plane_x name="p{m_.group(1)}" x="{int(m_.group(1)) * w!r}"/>', txt)
        open(d + "/input.xml", "w").write(txt)
        p = mc.Problem(d)
        par = p.lr_params()
        g, gs, r, rs = p.backward_density(par, 2_000_000, seed=5)
        g2, gs2 = p.backward(par, 2_000_000, seed=5)
        p.close()
    assert np.array_equal(g, g2) and np.array_equal(gs, gs2)
    ss, sa = par[0::2], par[1::2]
    combo = ss * g[0, 0::2] + sa * g[0, 1::2]
    assert np.allclose(r[0], combo, rtol=1e-9, atol=1e-15)
    assert np.all(rs[0] > 0)
    for reg in (0, 7, 15):
        h = 1e-4
        up_s, up_a, dn_s, dn_a = ss.copy(), sa.copy(), ss.copy(), sa.copy()
        up_s[reg] *= 1 + h
        up_a[reg] *= 1 + h
        dn_s[reg] *= 1 - h
        dn_a[reg] *= 1 - h
        tu = solve_slab([w] * R, up_s + up_a, up_s, n_mu=48, dx_max=0.0125)["transmission"]
        td = solve_slab([w] * R, dn_s + dn_a, dn_s, n_mu=48, dx_max=0.0125)["transmission"]
        exact = (tu - td) / (2 * h)
        assert abs(r[0, reg] - exact) <= 4 * rs[0, reg] + 1e-3 * abs(exact), (reg, r[0, reg], exact, rs[0, reg])
