"""The request stream's packing policy (piranha_gb300.stream.plan_packs), on
the CPU: every request is served exactly once, a pack holds one model's
requests within the image cap, its bucket holds it with at most a third of
padding, and packs open in arrival order."""
import numpy as np

from piranha_gb300 import stream


def _requests(n, seed):
    rng = np.random.default_rng(seed)
    return [("secureml" if rng.integers(0, 2) == 0 else "vgg16", int(rng.integers(1, 65))) for _ in range(n)]


def test_every_request_once_and_within_the_cap():
    reqs = _requests(512, 1)
    packs = stream.plan_packs(reqs, cap=128, lookahead=16)
    seen = sorted(r for p in packs for r in p.requests)
    assert seen == list(range(len(reqs)))
    heads = [p.requests[0] for p in packs]
    assert heads == sorted(heads)
    for p in packs:
        assert all(reqs[r][0] == p.model for r in p.requests)
        assert p.images == sum(reqs[r][1] for r in p.requests) <= 128
        assert p.bucket >= p.images and p.bucket in stream.BUCKETS
        assert p.requests == sorted(p.requests)
    # packing serves far fewer replays than requests
    assert len(packs) < len(reqs) / 2


def test_no_lookahead_is_one_request_per_pack():
    reqs = _requests(40, 2)
    packs = stream.plan_packs(reqs, cap=128, lookahead=0)
    assert [p.requests for p in packs] == [[i] for i in range(len(reqs))]
    assert all(p.bucket == stream.bucket_for(reqs[i][1]) for i, p in enumerate(packs))


def test_buckets_pad_at_most_a_third():
    for b in range(1, 129):
        k = stream.bucket_for(b)
        assert k >= b and (k - b) <= max(1, k // 3)


def test_choose_bucket_takes_a_faster_larger_bucket():
    # 112 images replay slower than 128 (rectangle vs position-major tiles)
    times = {64: 5.9e-3, 112: 11.0e-3, 128: 10.3e-3}
    assert stream.choose_bucket(times, 112) == 128
    assert stream.choose_bucket(times, 64) == 64       # a larger bucket that is slower is not taken
    assert stream.choose_bucket(times, 128) == 128
    # within the 3 % margin the pack stays on its own bucket
    assert stream.choose_bucket({112: 10.5e-3, 128: 10.3e-3}, 112) == 112
    # an untimed bucket is kept
    assert stream.choose_bucket({128: 1.0}, 96) == 96
    # never a smaller bucket
    assert stream.choose_bucket({16: 1e-4, 32: 1.0}, 32) == 32
