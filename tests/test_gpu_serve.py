"""The served form: requests arriving at Poisson times over two resident data
sets (a small bent tube and a small cube) join ticks already running, on
two streams at once; every result must be the same as the same job run
alone in a batch of its own (bit for bit: the form's arithmetic does not
depend on the mix)."""
import numpy as np
import pytest

import serve
import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["bf16", "fp64"])
def test_served_results_equal_alone(prec):
    tube = synth.bent_tube_mesh(nc=8, nax=40)
    _, tframes = synth.womersley_frames(tube, nframes=serve.TUBE_FRAMES)
    mesh = synth.kuhn_cube_mesh(8, jitter=0.2, seed=0)
    cframes = [synth.abc_flow(mesh[0], k * 0.02) for k in range(16)]
    sites = {"tube": serve.tube_site(prec, tube=tube, frames=tframes, h=0.004),
             "cube": serve.cube_site(prec, mesh=mesh, frames=cframes, nframes=16, hbm_budget=3_000_000)}
    reqs = serve.poisson_requests(tube, rate=300.0, duration=0.4, seed=3, tracer_range=(50, 3000),
                                  ftle_edges=(5, 12), rt_seeds=400, rt_periods=0.5, ftle_T=0.2)
    kinds = {r.kind for r in reqs}
    assert kinds == {"tracers", "ftle", "residence"}, kinds
    summary = serve.serve(sites, reqs, keep_results=True, time_limit=300)
    assert summary["requests"] == len(reqs)
    assert summary["p50_ms"] <= summary["p99_ms"]
    for r in reqs:
        site = sites[r.site]
        b = site.batch
        jid = serve.submit(b, r.job)
        b.run()
        if r.kind == "ftle":
            a = b.ftle_result(jid)
            assert np.array_equal(a[0], r.result[0]) and np.array_equal(a[1], r.result[1])
        elif r.kind == "residence":
            assert np.array_equal(b.residence_result(jid), r.result)
        else:
            a = b.tracer_result(jid)
            for k in ("X", "eid", "left", "ldt"):
                assert np.array_equal(a[k], r.result[k]), k
        b.release(jid)
    for s in sites.values():
        s.close()
