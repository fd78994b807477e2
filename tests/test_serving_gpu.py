"""Reward serving loop: every request's result equals the oracle, and is bit-identical alone and in the mix."""

import numpy as np
import pytest

from helpers import assert_tree
from oracle import panoptic as opan
from oracle import prefix as opre

pytestmark = pytest.mark.gpu

C, THINGS = 133, 80
ISTHING = [c < THINGS for c in range(C)]
THRESHOLDS = (0.5, 0.75)


@pytest.fixture(scope="module")
def pe():
    import panoptic_evaluator_gb300 as pe
    return pe


@pytest.fixture(scope="module")
def workload():
    return make_workload()


def make_workload():
    """14 uneven panoptic images and 7 prefix sequences (every, and a few selected, checkpoints)."""
    from panoptic_evaluator_gb300 import synthetic
    rng = np.random.default_rng(41)
    panoptic = [synthetic.segmentation_one(7, i, side=(33, 150), slots=(10, 40), dets=(0, 0)) for i in range(14)]
    prefixes = []
    for i in range(7):
        image = synthetic.prefix_one(9, i, side=(20, 90), masks=int(rng.integers(1, 24)), slots=int(rng.integers(10, 30)))
        n = len(image.masks)
        points = sorted(set(rng.integers(0, n + 1, int(rng.integers(1, 5))).tolist())) if i % 2 else None
        prefixes.append((image, points))
    return panoptic, prefixes


def make_requests(pe, workload):
    from panoptic_evaluator_gb300.serving import PanopticRequest, PrefixRequest
    panoptic, prefixes = workload
    requests = [PanopticRequest(im.pred, im.pred_classes, im.target, im.target_classes, im.crowd) for im in panoptic]
    requests += [PrefixRequest(im.masks, im.classes, im.target, im.target_classes, im.crowd, checkpoints=points)
                 for im, points in prefixes]
    order = np.random.default_rng(5).permutation(len(requests))
    return [requests[i] for i in order]


def server(pe, **kwargs):
    from panoptic_evaluator_gb300.serving import RewardServer
    kwargs.setdefault("memory_budget", 256 << 20)
    return RewardServer(C, isthing=ISTHING, iou_thresholds=THRESHOLDS, **kwargs)


def expected(request):
    if request.kind == "panoptic":
        pred = request.blob.numpy()[request.span: request.span + 4 * request.hw].view(np.int32)
        target = request.blob.numpy()[: 4 * request.hw].view(np.int32)
        pq = opan.panoptic_quality(pred.reshape(1, *request.shape), request.pred_classes[None],
                                   target.reshape(1, *request.shape), request.target_classes[None],
                                   request.crowd[None].astype(bool), C)
        return dict(pq=pq[0])
    target = request.blob.numpy()[: 4 * request.hw].view(np.int32).reshape(request.shape)
    rows = request.blob.numpy()[request.span: request.span + request.n * request.pitch].reshape(request.n, request.pitch)
    masks = rows[:, : request.hw].reshape(request.n, *request.shape).astype(bool)
    snaps = opre.segmentation_prefixes([masks], [request.classes], target[None], request.target_classes[None],
                                       request.crowd[None].astype(bool), C, isthing=ISTHING,
                                       checkpoints=request.points, iou_thresholds=THRESHOLDS)[0]
    keep = ("All", "Things", "Stuff", "miou", "prefix", "instance")
    return dict(snapshots=[{k: s[k] for k in keep} for s in snaps])


def results_alone(pe, requests):
    with server(pe) as alone:
        return [alone.submit(r).result().values for r in requests]


def test_each_request_matches_the_oracle(pe, workload):
    requests = make_requests(pe, workload)
    for request, got in zip(requests, results_alone(pe, requests)):
        assert_tree(got, expected(request), request.kind)


def test_mixed_batches_are_bit_identical_to_alone(pe, workload):
    requests = make_requests(pe, workload)
    alone = results_alone(pe, requests)
    for kwargs in (dict(max_batch=64, streams=4), dict(max_batch=3, streams=2), dict(max_batch=5, streams=4)):
        srv = server(pe, **kwargs)
        srv.start()
        futures = [srv.submit(r) for r in requests]  # queued together: the scheduler batches them
        responses = [f.result() for f in futures]
        srv.stop()
        assert max(r.batch_size for r in responses) > 1
        for got, want in zip(responses, alone):
            assert_tree(got.values, want, "mixed", exact_float=True)


def test_admission_respects_the_memory_budget(pe, workload):
    requests = make_requests(pe, workload)
    probe = server(pe)
    sizes = [probe.footprint(r) for r in requests]
    budget = 3 * max(sizes)
    srv = server(pe, memory_budget=budget)
    with srv:
        responses = [f.result() for f in [srv.submit(r) for r in requests]]
    assert srv.peak_in_flight_bytes <= budget
    assert srv.batches >= 2
    for got, want in zip(responses, results_alone(pe, requests)):
        assert_tree(got.values, want, "budgeted", exact_float=True)
    tiny = server(pe, memory_budget=min(sizes) - 1)
    with tiny:
        with pytest.raises(ValueError, match="budget"):
            tiny.submit(requests[0]).result()


def test_batches_respect_byte_cap_and_release_the_arena(pe, workload):
    requests = make_requests(pe, workload)
    biggest = max(r.blob.numel() for r in requests)
    srv = server(pe, max_batch_bytes=biggest + 1)
    with srv:
        responses = [f.result() for f in [srv.submit(r) for r in requests]]
    assert srv._arena.used == 0 and srv._arena.free == [(0, srv._arena.nbytes)]
    for got, want in zip(responses, results_alone(pe, requests)):
        assert_tree(got.values, want, "byte-capped", exact_float=True)


def test_dataset_totals_follow_every_panoptic_request(pe, workload):
    requests = [r for r in make_requests(pe, workload) if r.kind == "panoptic"]
    srv = server(pe, max_batch=4)
    with srv:
        for f in [srv.submit(r) for r in requests]:
            f.result()
    tp = np.zeros(C, np.int64)
    fp = np.zeros(C, np.int64)
    fn = np.zeros(C, np.int64)
    sums = np.zeros(C)
    for r in requests:
        stats = opan.reward_statistics(
            r.blob.numpy()[r.span: r.span + 4 * r.hw].view(np.int32).reshape(1, *r.shape), r.pred_classes[None],
            r.blob.numpy()[: 4 * r.hw].view(np.int32).reshape(1, *r.shape), r.target_classes[None],
            r.crowd[None].astype(bool), C)
        sums += stats[0][0]
        tp += stats[1][0]
        fp += stats[2][0]
        fn += stats[3][0]
    assert_tree({k: v.cpu() for k, v in srv.totals.items()}, dict(tp=tp, fp=fp, fn=fn, iou_sum=sums))


def test_open_loop_poisson_run_reports_latency(pe, workload):
    from panoptic_evaluator_gb300.serving import serve
    requests = make_requests(pe, workload) * 3
    alone = results_alone(pe, requests[: len(requests) // 3]) * 3
    arrivals = np.cumsum(np.random.default_rng(3).exponential(1 / 2000.0, len(requests)))
    with server(pe, max_batch=8) as srv:
        responses, summary = serve(srv, requests, arrivals)
    assert summary["requests"] == len(requests) and summary["p99_ms"] >= summary["p50_ms"] > 0
    for got, want in zip(responses, alone):
        assert_tree(got.values, want, "poisson", exact_float=True)


def test_invalid_request_fails_only_its_batch(pe, workload):
    from panoptic_evaluator_gb300.serving import PanopticRequest
    im = workload[0][0]
    bad = PanopticRequest(im.pred, im.pred_classes, np.full_like(im.target, 10_000), im.target_classes, im.crowd)
    srv = server(pe, validate=True)
    with srv:
        with pytest.raises(ValueError):
            srv.submit(bad).result()
        good = srv.submit(PanopticRequest(im.pred, im.pred_classes, im.target, im.target_classes, im.crowd)).result()
    assert_tree(good.values, expected(PanopticRequest(im.pred, im.pred_classes, im.target, im.target_classes,
                                                      im.crowd)))


def test_cancelled_requests_are_dropped_and_the_rest_served(pe, workload):
    """A request cancelled while queued is never run; the others are served with their exact results."""
    requests = make_requests(pe, workload)
    srv = server(pe)
    futures = [srv.submit(r) for r in requests]  # queued before the scheduler starts
    cancelled = [f.cancel() for f in futures[::3]]
    assert all(cancelled)
    with srv:
        kept = [(r, f) for i, (r, f) in enumerate(zip(requests, futures)) if i % 3]
        results = [(r, f.result(timeout=60)) for r, f in kept]
    assert all(f.cancelled() for f in futures[::3])
    for request, response in results:
        assert_tree(response.values, expected(request))
