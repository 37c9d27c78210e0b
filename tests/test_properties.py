"""Property tests (hypothesis) of the oracle and of the library's host-side conventions, on the
CPU: the kept-mode counts of the 2/3 rule against the library's own, dealiasing and the divergence
corrections as projections, linearity of the diffusion and penalty terms, and the retained band
of the right-hand side depending on the retained band of the state only."""
import functools
import inspect
import random

import numpy as np

try:
    from hypothesis import given, settings
    from hypothesis import strategies as st

    SETTINGS = settings(max_examples=12, deadline=None)
except ImportError:  # hosts without hypothesis run the same properties on fixed seeded draws
    class _Strategy:
        def __init__(self, draw):
            self.draw = draw

        def filter(self, pred):
            def draw(rng):
                while True:
                    v = self.draw(rng)
                    if pred(v):
                        return v
            return _Strategy(draw)

    class st:  # noqa: N801 - the subset of hypothesis.strategies used here
        integers = staticmethod(lambda min_value, max_value: _Strategy(lambda rng: rng.randint(min_value, max_value)))
        sampled_from = staticmethod(lambda xs: _Strategy(lambda rng: rng.choice(list(xs))))
        floats = staticmethod(lambda lo, hi: _Strategy(lambda rng: rng.uniform(lo, hi)))

    def given(*strategies):
        def wrap(fn):
            names = list(inspect.signature(fn).parameters)[-len(strategies):]
            fixtures = list(inspect.signature(fn).parameters)[:-len(strategies)]

            @functools.wraps(fn)
            def run(**kw):
                rng = random.Random(fn.__name__)
                for _ in range(12):
                    fn(**kw, **{nm: s.draw(rng) for nm, s in zip(names, strategies)})

            run.__signature__ = inspect.Signature([inspect.Parameter(f, inspect.Parameter.POSITIONAL_OR_KEYWORD)
                                                   for f in fixtures])
            return run
        return wrap

    def SETTINGS(fn):  # noqa: N802
        return fn


@SETTINGS
@given(st.integers(min_value=4, max_value=1024).filter(lambda n: n % 2 == 0))
def test_kept_counts_match_library(pkg, mo, n):
    kx, kp, kn = pkg.kept_modes(n)
    assert (kx, kp, kn) == mo.kept_counts(n)
    assert kx == kp and 0 <= kn <= kp <= n // 2  # the rfft axis keeps exactly the kept non-negative modes
    assert kp + kn <= n


def _spectrum(rng, g):
    return rng.standard_normal((6, g.n, g.n, g.nkr)) + 1j * rng.standard_normal((6, g.n, g.n, g.nkr))


@SETTINGS
@given(st.sampled_from([8, 12, 16]), st.integers(0, 2 ** 31 - 1))
def test_dealias_and_div_correct_are_projections(mo, n, seed):
    g = mo.Grid(n)
    rng = np.random.default_rng(seed)
    a = _spectrum(rng, g)
    d = g.dealias(a.copy())
    assert np.array_equal(g.dealias(d.copy()), d)
    c = mo.div_correct(g, d.copy(), 3)
    assert np.allclose(mo.div_correct(g, c.copy(), 3), c, rtol=0, atol=1e-12 * np.abs(c).max())
    ks = g.ks
    for off in (0, 3):
        kdot = sum(ks[i] * c[off + i] for i in range(3))
        assert np.abs(kdot).max() <= 1e-10 * np.abs(c).max()


@SETTINGS
@given(st.sampled_from([8, 12]), st.integers(0, 2 ** 31 - 1), st.floats(1e-4, 1e-1), st.floats(1e-4, 1e-1))
def test_diffusion_is_linear_in_viscosity(mo, n, seed, nu, eta):
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=seed % 1000)
    base, a = np.zeros_like(s), np.zeros_like(s)
    mo.calcN_fast(base, s.copy(), g, 0.0, 0.0)
    mo.calcN_fast(a, s.copy(), g, nu, eta)
    g.dealias(s)
    H = mo.hermitian_kx0(g, s)
    expect = base.copy()
    expect[:3] -= g.Krsq * nu * H[:3]
    expect[3:] -= g.Krsq * eta * H[3:]
    assert np.allclose(a, expect, rtol=1e-12, atol=1e-12 * np.abs(expect).max())


@SETTINGS
@given(st.sampled_from([8, 12]), st.integers(0, 2 ** 31 - 1), st.floats(0.1, 10.0))
def test_penalty_scales_with_the_mask(mo, n, seed, c):
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=seed % 1000)
    x, y, z = g.mesh()
    chi = 0.5 * (1 + np.sin(x) * np.cos(y + z))
    plain, one, scaled = np.zeros_like(s), np.zeros_like(s), np.zeros_like(s)
    mo.calcN_fast(plain, s.copy(), g, 1e-3, 1e-3)
    mo.calcN_fast(one, s.copy(), g, 1e-3, 1e-3, vp=dict(chi=chi, dt=1e-3))
    mo.calcN_fast(scaled, s.copy(), g, 1e-3, 1e-3, vp=dict(chi=c * chi, dt=1e-3))
    assert np.allclose(scaled - plain, c * (one - plain), rtol=1e-10, atol=1e-10 * np.abs(one - plain).max())


@SETTINGS
@given(st.sampled_from([8, 12]), st.integers(0, 2 ** 31 - 1))
def test_rhs_ignores_the_alias_band_of_the_state(mo, n, seed):
    g = mo.Grid(n)
    rng = np.random.default_rng(seed)
    s = mo.random_spectrum_state(g, seed=seed % 1000)
    noisy = s + 1e3 * _spectrum(rng, g) * (~g.retained_mask())
    a, b = np.zeros_like(s), np.zeros_like(s)
    mo.calcN_literal(a, s.copy(), g, 1e-3, 2e-3)
    mo.calcN_literal(b, noisy.copy(), g, 1e-3, 2e-3)
    m = g.retained_mask()
    assert np.allclose(a[:, m], b[:, m], rtol=1e-12, atol=1e-12 * np.abs(a).max())
