"""Request loop: factor-of-safety solves of different meshes admitted by HBM
footprint and run concurrently; each result is the same alone and in the mix."""
import numpy as np
import pytest

import specfem3d_geotech_gb300 as sg
from specfem3d_geotech_gb300 import meshgen

pytestmark = pytest.mark.gpu


def requests(n=4, seed=4):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(200), np.log(800), n)).astype(int)
    return [meshgen.random_slope(rng, int(s)) for s in sizes]


def control():
    # a short plastic-iteration cap keeps the test quick; the semantics are the reference's
    return sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=60, precision=sg.PREC_MIXED)


def test_results_same_alone_and_in_the_mix(ctx):
    reqs = requests()
    ctl = control()
    alone = []
    for m in reqs:
        model = sg.Model(m, precision=sg.PREC_MIXED, ctx=ctx)
        alone.append(model.fos(ctl, lo=1.0, hi=2.0, step=0.1, k=4))
        model.close()
    srv = sg.Server(0, 0, workers=4)
    ids = [srv.submit(m, ctl, lo=1.0, hi=2.0, step=0.1, k=4) for m in reqs]
    got = [srv.wait(i, timeout=600) for i in ids]
    st = srv.stats()
    srv.close()
    for a, g in zip(alone, got):
        assert g["status"] == 0
        assert g["fos"] == a[0] and g["ntrials"] == a[1] and g["nrounds"] == a[2]
    assert st["completed"] == len(reqs)
    assert st["peak_concurrent"] >= 2           # the requests overlapped on the device
    assert st["p99_s"] >= st["p50_s"] > 0


def test_admission_by_hbm_footprint(ctx):
    """A budget that holds one request at a time serialises them; none fails."""
    mesh = requests(1, seed=5)[0]
    ctl = control()
    srv0 = sg.Server(0, 0, workers=1)
    r0 = srv0.wait(srv0.submit(mesh, ctl, lo=1.0, hi=2.0, step=0.1, k=4), timeout=600)
    srv0.close()
    budget = int(r0["footprint"] * 1.5)
    srv = sg.Server(0, budget, workers=3)
    ids = [srv.submit(mesh, ctl, lo=1.0, hi=2.0, step=0.1, k=4) for _ in range(3)]
    got = [srv.wait(i, timeout=600) for i in ids]
    st = srv.stats()
    srv.close()
    assert all(g["status"] == 0 and g["fos"] == r0["fos"] for g in got)
    assert st["peak_concurrent"] == 1
    # arrival-order admission: each starts after the previous one finished
    for a, b in zip(got, got[1:]):
        assert b["t_start"] >= a["t_done"] - 1e-3


def test_excavation_requests_in_the_mix(ctx):
    """Staged-excavation requests admitted beside factor-of-safety requests
    give the same stage results as the same excavation run alone, and the
    mixed requests overlap on the device."""
    exc = meshgen.excavation(nx=6, ny=6, nz=4, L=12.0, H=8.0, pit=4.0, lifts=2, lift_h=2.0)
    ctl64 = sg.make_control(cg_tol=1e-8, nl_tol=1e-4, cg_maxiter=5000, nl_maxiter=200)
    model = sg.Model(exc, ctx=ctx)
    alone = model.excavation(ctl64, 1, 8.0, 0.0, 0.5, [2, 3])
    model.close()
    slopes = requests(2, seed=6)
    ctl = control()
    srv = sg.Server(0, 0, workers=3)
    ids = [srv.submit(slopes[0], ctl, lo=1.0, hi=2.0, step=0.1, k=4),
           srv.submit_excavation(exc, ctl64, 1, 8.0, 0.0, 0.5, [2, 3]),
           srv.submit(slopes[1], ctl, lo=1.0, hi=2.0, step=0.1, k=4)]
    got = [srv.wait(i, timeout=600) for i in ids]
    st = srv.stats()
    srv.close()
    g = got[1]
    assert g["status"] == 0 and g["kind"] == 1 and g["nstage"] == alone.shape[0]
    assert np.array_equal(g["stages"], alone)          # same device code, same order: bitwise
    assert g["ntrials"] == int(alone[:, 2].sum())
    assert all(r["status"] == 0 and r["kind"] == 0 for r in (got[0], got[2]))
    assert st["completed"] == 3 and st["peak_concurrent"] >= 2
