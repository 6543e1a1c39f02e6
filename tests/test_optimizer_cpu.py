"""Host-side parameter search without a GPU: the library's Nelder-Mead
(cafe_nelder_mead) against the reference's fminsearch_min on analytic
objectives, and the discrete-gamma categories against get_gamma. Both are
plain FP64 host arithmetic compiled without contraction, so the bar is
bit-exact: same best point, score, iteration and evaluation counts."""
import ctypes as C
import math

import numpy as np
import pytest

from golden_cases import load_json


@pytest.fixture(scope="module")
def lib():
    from cafe5_gb300 import _lib, build
    build.build()
    return _lib.load()


def objective(fn):
    """The harness's analytic objectives, same expressions and order."""
    def f(xp, n, _user):
        x = [xp[i] for i in range(n)]
        if fn in ("rosen", "wall"):
            if fn == "wall" and x[0] > 1.0:
                return math.inf
            s = 0.0
            for i in range(n - 1):
                a = x[i + 1] - x[i] * x[i]
                b = 1 - x[i]
                s += 100 * a * a + b * b
            return s
        if fn == "bowl":
            s = 0.0
            for i in range(n):
                d = x[i] - (i + 1)
                s += d * d * (i + 1)
            return s
        s = 1.0
        for v in x:
            s *= v
        return s
    return f


def search(lib, fn, x0, max_iterations):
    from cafe5_gb300 import _lib
    x = np.ascontiguousarray(x0, dtype=np.float64)
    best = np.zeros(len(x))
    cfg = _lib.OptConfig(_lib.OPT_LAMBDA, len(x), x.ctypes.data, max_iterations, 0.0, 0.0)
    res = _lib.OptResult(best.ctypes.data, 0.0, 0, 0, 0)
    cb = _lib.OBJECTIVE(objective(fn))
    assert lib.cafe_nelder_mead(C.byref(cfg), cb, None, C.byref(res)) == 0
    return best, res


@pytest.mark.parametrize("g", load_json("ref_optimizer.json")["analytic"],
                         ids=lambda g: f"{g['objective']}-{len(g['initial'])}d-{g['max_iterations']}")
def test_nelder_mead_matches_reference_bits(lib, g):
    best, res = search(lib, g["objective"], g["initial"], g["max_iterations"])
    assert [v.hex() for v in best] == [float.fromhex(h).hex() for h in g["best_hex"]]
    assert res.score.hex() == float.fromhex(g["score_hex"]).hex()
    assert res.iterations == g["iters"]
    assert res.evaluations == g["evals"]
    assert res.converged == (1 if g["iters"] < g["max_iterations"] else 0)


def test_nelder_mead_initial_simplex_known_answer(lib):
    """test.cpp:2864-2882 (fminsearch_min_init with the multiplier scorer,
    X0 = {5, 3}): the first vertex scores 15, the next best 15.75. One
    iteration is run; with the product objective its first reflection is
    scored against those vertices."""
    seen = []

    def f(xp, n, _u):
        v = xp[0] * xp[1]
        seen.append(v)
        return v
    from cafe5_gb300 import _lib
    x = np.array([5.0, 3.0])
    best = np.zeros(2)
    cfg = _lib.OptConfig(0, 2, x.ctypes.data, 1, 0.0, 0.0)
    res = _lib.OptResult(best.ctypes.data, 0.0, 0, 0, 0)
    cb = _lib.OBJECTIVE(f)
    assert lib.cafe_nelder_mead(C.byref(cfg), cb, None, C.byref(res)) == 0
    assert sorted(seen[:3])[:2] == [15.0, 15.75]


def test_nelder_mead_rejects_bad_arguments(lib):
    from cafe5_gb300 import _lib
    best = np.zeros(1)
    res = _lib.OptResult(best.ctypes.data, 0.0, 0, 0, 0)
    cfg = _lib.OptConfig(0, 0, None, 0, 0.0, 0.0)
    cb = _lib.OBJECTIVE(lambda xp, n, u: 0.0)
    assert lib.cafe_nelder_mead(C.byref(cfg), cb, None, C.byref(res)) == 6
    assert lib.cafe_optimize(None, None, None, None) == 6


def test_discrete_gamma_bits_match_reference(lib):
    from cafe5_gb300.inputs import discrete_gamma
    for g in load_json("ref_matrices.json")["gamma"]:
        probs, mult = discrete_gamma(g["alpha"], g["K"])
        assert [m.hex() for m in mult] == [float.fromhex(x).hex() for x in g["multipliers"]], (g["K"], g["alpha"])
        assert probs == [float.fromhex(x) for x in g["probs"]]


def test_discrete_gamma_properties(lib):
    """Multipliers average 1 and increase; a single category is rate 1;
    alpha <= 0 is refused (gamma_model::can_infer rejects alpha < 0)."""
    from cafe5_gb300.inputs import discrete_gamma
    for a in (0.05, 0.3, 1.0, 4.0, 50.0):
        for K in (2, 3, 5, 10):
            p, m = discrete_gamma(a, K)
            assert abs(sum(m) / K - 1) < 1e-12
            assert all(m[i] < m[i + 1] for i in range(K - 1))
            assert p == [1.0 / K] * K
    assert discrete_gamma(0.7, 1) == ([1.0], [1.0])
    with pytest.raises(ValueError):
        discrete_gamma(-0.5, 4)
