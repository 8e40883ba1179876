"""GPU: the request loop (continuous batching).  Every request's receivers
must equal a standalone run of the same set-up, alone or in the mix, and the
HBM budget must bound how many requests run at once.  Rooms whose x extent is
not a multiple of 16 run on a domain padded with outside nodes (the
standalone runs are not padded), so the comparison also checks that the
padding leaves every receiver unchanged."""
import numpy as np
import pytest

from parallelfdtd_gb300 import _lib as L
from parallelfdtd_gb300 import materials, rooms
from parallelfdtd_gb300.domain import Domain, default_params
from parallelfdtd_gb300.serving import DONE, FAILED, Request, Server, build_request, \
    run_trace, serving_trace

pytestmark = pytest.mark.gpu

# (dims, steps, fields, precision, scheme, dif, tb)
SPECS = [((48, 40, 36), 220, 1, "f32", "forward", False, 0),
         ((64, 48, 40), 180, 4, "f32", "iwb", True, 0),
         ((40, 56, 44), 260, 2, "f16", "centred", True, 0),
         ((56, 44, 40), 200, 1, "f64", "forward", True, 0),
         ((72, 64, 48), 150, 4, "bf16", "forward", False, 2),
         ((44, 44, 60), 240, 1, "f32", "iwb", False, 0)]


def spec_inputs(i, spec):
    dims, steps, fields, prec, scheme, dif, tb = spec
    room = rooms.boxes_room(dims, n_boxes=4, edge=(4, 12), n_materials=5, seed=40 + i)
    n_src = fields
    pts = room.random_air_nodes(3 * n_src, seed=50 + i)
    srcs = [tuple(p) for p in pts[:n_src]]
    recs = [tuple(p) for p in pts[n_src:]]
    pulse = rooms.gaussian_pulse(steps, 3.0)
    samples = np.stack([pulse * (1 + 0.2 * f) for f in range(n_src)])
    d = None
    if dif:
        d = (np.array([m % 2 for m in range(5)], np.int32),
             materials.dif_table(materials.positive_real_filters(5, 3, seed=60 + i), 3))
    return room, srcs, recs, samples, d


def make_request(i, spec):
    dims, steps, fields, prec, scheme, dif, tb = spec
    room, srcs, recs, samples, d = spec_inputs(i, spec)
    return Request.from_room(room, steps, srcs, recs, samples, precision=prec, scheme=scheme,
                             fields=fields, src_fields=list(range(fields)),
                             rec_fields=[j // 2 for j in range(2 * fields)], dif=d, tb=tb)


def alone(i, spec):
    dims, steps, fields, prec, scheme, dif, tb = spec
    room, srcs, recs, samples, d = spec_inputs(i, spec)
    with Domain(dims, prec, fields=fields) as dom:
        dom.set_voxels(room.bid, room.mat, centred=(scheme != "forward"))
        dom.set_materials(room.admittance)
        if d is not None:
            dom.set_dif_filters(*d)
        dom.set_params(default_params(scheme=scheme))
        dom.set_scheme(scheme)
        dom.set_sources(srcs, [1] * fields, samples, fields=list(range(fields)))
        dom.set_receivers(recs, fields=[j // 2 for j in range(2 * fields)])
        dom.set_temporal_block(tb)
        g, _, st = dom.run(steps)
        assert st == 0
    return g


def test_mix_equals_alone(gpu):
    ref = [alone(i, s) for i, s in enumerate(SPECS)]
    with Server(0, hbm_budget=8 << 30, max_active=4) as srv:
        tickets = [srv.submit(make_request(i, s)) for i, s in enumerate(SPECS)]
        for i, t in enumerate(tickets):
            assert srv.wait(t, 120.0) == DONE, srv.error(t)
            out, times = srv.result(t)
            assert np.abs(ref[i]).max() > 0
            assert np.array_equal(out, ref[i]), f"request {i} differs in the mix"
            assert times[0] >= 0 and times[1] > 0 and abs(times[2] - times[0] - times[1]) < 1e-6
        st = srv.stats()
    assert st["completed"] == len(SPECS) and st["failed"] == 0
    assert st["max_running"] >= 2, "requests never overlapped"
    assert st["bytes_in_use"] == 0


def test_budget_bounds_concurrency(gpu):
    """A budget that holds any one of the requests but no two runs them one at
    a time."""
    idx = [0, 1, 2, 3]
    reqs = [make_request(i, SPECS[i]) for i in idx]
    sizes = sorted(r.bytes() for r in reqs)
    budget = int(1.2 * sizes[-1])
    assert budget < sizes[0] + sizes[1]
    with Server(0, hbm_budget=budget, max_active=8) as srv:
        tickets = [srv.submit(r) for r in reqs]
        srv.drain(120.0)
        for i, t in zip(idx, tickets):
            out, _ = srv.result(t)
            assert np.array_equal(out, alone(i, SPECS[i]))
        st = srv.stats()
    assert st["max_running"] == 1
    assert st["bytes_peak"] <= budget


def test_oversize_request_fails(gpu):
    req = make_request(0, SPECS[0])
    with Server(0, hbm_budget=1 << 20, max_active=2) as srv:
        with pytest.raises(L.PfdtdError):
            srv.submit(req)
        assert srv.stats()["failed"] == 1


def test_small_trace(gpu):
    trace = serving_trace(6, seed=3, rate=50.0, axis=(40, 96), steps=(100, 300), sources=(1, 4))
    reqs = [build_request(it) for it in trace]
    with Server(0, hbm_budget=16 << 30, max_active=4) as srv:
        res = run_trace(srv, reqs, [it.arrival for it in trace], timeout=300.0)
    assert res["stats"]["completed"] == 6
    assert res["latency_p99_s"] >= res["latency_p50_s"] > 0
    assert res["throughput"] > 0


def test_iwb_fields_run_apart(gpu):
    """An IWB request with 4 fields and sources on fields 0 and 2 only runs
    those two fields one after the other on one single-field domain (the
    single-field IWB kernels); its receivers equal a batched run of the same
    set-up bit for bit, and the receivers of the fields without a source stay
    0.  Two such requests run at once, so parts of different requests
    interleave."""
    from parallelfdtd_gb300 import materials
    dims, steps = (100, 44, 40), 160
    room = rooms.boxes_room(dims, n_boxes=4, edge=(4, 12), n_materials=5, seed=71)
    pts = room.random_air_nodes(10, seed=72)
    srcs, recs = [tuple(p) for p in pts[:2]], [tuple(p) for p in pts[2:10]]
    src_fields, rec_fields = [0, 2], [0, 0, 1, 1, 2, 2, 3, 3]
    pulse = rooms.gaussian_pulse(steps, 3.0)
    samples = np.stack([pulse, -0.7 * pulse])
    dif = (np.array([m % 2 for m in range(5)], np.int32),
           materials.dif_table(materials.positive_real_filters(5, 3, seed=73), 3))
    with Domain(dims, "f32", fields=4) as dom:
        dom.set_voxels(room.bid, room.mat, centred=True)
        dom.set_materials(room.admittance)
        dom.set_dif_filters(*dif)
        dom.set_params(default_params(scheme="iwb"))
        dom.set_scheme("iwb")
        dom.set_sources(srcs, [1, 1], samples, fields=src_fields)
        dom.set_receivers(recs, fields=rec_fields)
        ref, _, st = dom.run(steps)
        assert st == 0
    req = Request.from_room(room, steps, srcs, recs, samples, precision="f32", scheme="iwb",
                            fields=4, src_fields=src_fields, rec_fields=rec_fields, dif=dif)
    assert req.computed_updates() == req.node_updates()
    req2 = Request.from_room(room, steps, srcs, recs, samples, precision="f32", scheme="iwb",
                             fields=4, src_fields=src_fields, rec_fields=rec_fields, dif=dif)
    with Server(0, hbm_budget=8 << 30, max_active=2) as srv:
        tickets = [srv.submit(req), srv.submit(req2)]
        outs = []
        for t in tickets:
            assert srv.wait(t, 120.0) == DONE, srv.error(t)
            outs.append(srv.result(t)[0])
        st = srv.stats()
    assert st["completed"] == 2 and st["admitted"] == 2 and st["bytes_in_use"] == 0
    assert np.abs(ref[[0, 1, 4, 5]]).max() > 1e-4
    assert (ref[[2, 3, 6, 7]] == 0).all()
    for out in outs:
        assert np.array_equal(out, ref)
