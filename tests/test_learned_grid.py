"""Learned per-centre radial grids (inca_parallel_gb300/learned_grid.py), CPU parts: the 1D
radial quadrature objective, the training targets and the numpy reference of the network that
checks the GPU kernels (its gradient against finite differences, float64, 1e-6 relative)."""
import math

import numpy as np

from inca_parallel_gb300 import learned_grid as LG


def test_radial_rule_converges():
    errs = [LG.radial_errors([1.0], [1.0], n)[0, 0] for n in (10, 20, 40, 75)]
    assert errs[0] > errs[-1]
    assert errs[-1] < 1e-12


def test_best_scale_beats_the_reference_scale():
    e = np.array([0.3, 2.0, 40.0, 900.0])
    a = 1.2
    base = LG.radial_errors([a], e, 30).mean()
    s, best = LG.best_scale(e, 30, a)
    assert best <= base
    assert 1.2 / 8 <= s <= 1.2 * 8


def test_features_and_targets():
    from inca_parallel_gb300 import centercalc, workloads as W
    rng = np.random.default_rng(2)
    b = W.random_molecule(rng, 5, 25)
    cent, Ps, alf = centercalc(b["an"], b["cartes"])
    F, E = LG.features(b, cent, Ps, alf, 30)
    assert F.shape == (len(Ps), LG.NFEAT) and np.isfinite(F).all()
    T = LG.targets(E, alf, 30)
    assert T.shape == (len(Ps), 2) and np.isfinite(T).all()
    assert np.all(np.exp(T[:, 1]) >= 10) and np.all(np.exp(T[:, 1]) <= LG.NRAD_MAX)


def test_reference_network_gradient_by_finite_differences():
    rng = np.random.default_rng(4)
    nin, nh, nout = 5, 7, 2
    npar = nh * nin + nh + nh * nh + nh + nout * nh + nout
    p = rng.normal(scale=0.5, size=npar)
    X = rng.normal(size=(11, nin))
    T = rng.normal(size=(11, nout))
    _, loss, g = LG.mlp_reference(p, nin, nh, nout, X, T)
    h = 1e-6
    for i in rng.choice(npar, 25, replace=False):
        q = p.copy()
        q[i] += h
        lp = LG.mlp_reference(q, nin, nh, nout, X, T)[1]
        q[i] -= 2 * h
        lm = LG.mlp_reference(q, nin, nh, nout, X, T)[1]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])
    assert math.isfinite(loss)
