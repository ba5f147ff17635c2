"""Serving loop (pgpu_server_*): results of requests run in a concurrent mix equal the same
requests run alone through Interpolant (same kernels, same order of operations), admission
keeps the charged device bytes within the budget, and failures are reported per request."""
import numpy as np
import pytest

import polatory_gb300 as pg
from polatory_gb300 import _lib, workloads

pytestmark = pytest.mark.gpu


def models():
    cov = pg.Model(pg.CovExponential([1.0, 0.3]), 0)
    cov.nugget = 1e-3
    return [
        pg.Model(pg.Biharmonic3D([1.0]), 1),
        pg.Model(pg.Triharmonic3D([1.0]), 1),
        cov,
        pg.Model(pg.Biharmonic3D([1.0]), 0),
    ]


def problem(seed, n):
    g = np.random.Generator(np.random.PCG64(seed))
    p = g.random((n, 3))
    v = workloads.f_c1(p) + g.normal(0.0, 1e-4, n)
    return p, v


def test_results_same_alone_and_in_the_mix():
    ms = models()
    probs = [problem(100 + i, 1500 + 700 * i) for i in range(len(ms))]
    g = np.random.Generator(np.random.PCG64(7))
    queries = [g.random((400 + 150 * i, 3)) for i in range(6)]
    tol = 1e-5

    alone = {}
    for k, (m, (p, v)) in enumerate(zip(ms, probs)):
        it = pg.Interpolant(m)
        it.fit(p, v, tol)
        alone[k] = [it.evaluate(q) for q in queries]

    with pg.Server(n_workers=6) as s:
        fits, evals = [], []
        # Unrelated fits in other slots keep the workers busy around the checked requests.
        noise = [s.submit_fit(10 + i, ms[i % 4], *problem(200 + i, 2500), tol) for i in range(4)]
        for k, m in enumerate(ms):
            fits.append(s.submit_fit(k, m, *probs[k], tol))
        for rep in range(2):
            for k in range(len(ms)):
                for j, q in enumerate(queries):
                    evals.append((k, j, s.submit_evaluate(k, q)))
        for t in noise + fits:
            st, lat, _, msg = s.wait(t)
            assert st == 0, msg
            assert lat > 0
        for k, j, t in evals:
            st, _, out, msg = s.wait(t)
            assert st == 0, msg
            np.testing.assert_array_equal(out, alone[k][j])
        stats = s.stats()
        assert stats["completed"] == len(noise) + len(fits) + len(evals)
        assert stats["failed"] == 0
        assert stats["peak_bytes"] <= stats["budget_bytes"]


def test_evaluation_reads_the_fit_submitted_before_it():
    m = pg.Model(pg.Biharmonic3D([1.0]), 1)
    p1, v1 = problem(1, 2000)
    p2, v2 = problem(2, 2600)
    q = np.random.Generator(np.random.PCG64(3)).random((300, 3))
    want = []
    for p, v in ((p1, v1), (p2, v2)):
        it = pg.Interpolant(m)
        it.fit(p, v, 1e-5)
        want.append(it.evaluate(q))
    with pg.Server(n_workers=4) as s:
        t1 = s.submit_fit(0, m, p1, v1, 1e-5)
        e1 = s.submit_evaluate(0, q)
        t2 = s.submit_fit(0, m, p2, v2, 1e-5)
        e2 = s.submit_evaluate(0, q)
        for t in (t1, t2):
            assert s.wait(t)[0] == 0
        np.testing.assert_array_equal(s.wait(e1)[2], want[0])
        np.testing.assert_array_equal(s.wait(e2)[2], want[1])


def test_slot_holds_latest_fit_when_fits_finish_out_of_order():
    m = pg.Model(pg.Biharmonic3D([1.0]), 1)
    big = problem(11, 20000)
    small = problem(12, 1000)
    q = np.random.Generator(np.random.PCG64(13)).random((200, 3))
    it = pg.Interpolant(m)
    it.fit(*small, 1e-5)
    want = it.evaluate(q)
    with pg.Server(n_workers=4) as s:
        t1 = s.submit_fit(0, m, *big, 1e-5)    # finishes last
        t2 = s.submit_fit(0, m, *small, 1e-5)  # submitted last: the slot's model
        assert s.wait(t2)[0] == 0
        assert s.wait(t1)[0] == 0
        st, _, out, msg = s.wait(s.submit_evaluate(0, q))
        assert st == 0, msg
        np.testing.assert_array_equal(out, want)


def test_admission_within_budget():
    m = pg.Model(pg.Biharmonic3D([1.0]), 1)
    one = pg.Server.estimate_bytes(_lib.REQUEST_FIT, 3000)
    budget = int(one * 2.5)  # at most two fits of this size in flight
    with pg.Server(n_workers=8, hbm_budget_bytes=budget) as s:
        ts = [s.submit_fit(i, m, *problem(300 + i, 3000), 1e-5) for i in range(8)]
        for t in ts:
            assert s.wait(t)[0] == 0
        st = s.stats()
        assert st["peak_bytes"] <= budget
        assert st["completed"] == 8


def test_oversize_request_rejected():
    m = pg.Model(pg.Biharmonic3D([1.0]), 1)
    with pg.Server(n_workers=2, hbm_budget_bytes=1 << 20) as s:
        with pytest.raises(pg.PolatoryError) as e:
            s.submit_fit(0, m, *problem(5, 1000), 1e-5)
        assert e.value.code == _lib.PGPU_REJECTED
        assert s.stats()["rejected"] == 1


def test_failures_reported_per_request():
    m = pg.Model(pg.Triharmonic3D([1.0]), 1)
    with pg.Server(n_workers=2) as s:
        with pytest.raises(pg.PolatoryError):
            s.submit_evaluate(3, np.zeros((4, 3)))  # slot holds no model
        t = s.submit_fit(0, m, *problem(9, 3000), 1e-13, max_iter=1)
        e = s.submit_evaluate(0, np.zeros((4, 3)))
        ok = s.submit_fit(1, m, *problem(10, 1000), 1e-5)
        st, _, _, msg = s.wait(t)
        assert st != 0 and msg
        assert s.wait(e)[0] != 0
        assert s.wait(ok)[0] == 0
