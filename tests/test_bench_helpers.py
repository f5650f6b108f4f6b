"""bench.py's host-side pieces that need no GPU: the batch workload's
definition (so measurements of different builds stay comparable), the
reference arm's sample (the whole batch), and the accuracy statistics."""
import hashlib
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_batch_workload_is_fixed():
    vs = bench.batch_views(bench.SEED)
    assert len(vs) == 64
    assert [v['algorithm'] for v in vs] == ['linkedlist', 'loop64'] * 32
    for v in vs:
        assert 256 <= v['width'] == v['height'] <= 2048
        assert 64 <= v['spheres'] <= 8192
        assert v['oit_layers'] in (4, 8, 16, 32)
    for alg in ('linkedlist', 'loop64'):  # every OIT_LAYERS value for both algorithms
        assert sorted({v['oit_layers'] for v in vs if v['algorithm'] == alg}) == [4, 8, 16, 32]
    # the same 64 views on every host and numpy version this project runs on
    digest = hashlib.sha256(json.dumps(vs, sort_keys=True).encode()).hexdigest()
    again = hashlib.sha256(json.dumps(bench.batch_views(bench.SEED), sort_keys=True).encode()).hexdigest()
    assert digest == again
    assert (min(v['width'] for v in vs), max(v['width'] for v in vs)) == (261, 1972)
    assert (min(v['spheres'] for v in vs), max(v['spheres'] for v in vs)) == (66, 7210)


def test_reference_arm_renders_the_whole_batch():
    """The reference arm's step is the GPU arm's step: all 64 views."""
    picked = bench.reference_views()
    assert len(picked) == 64
    key = lambda v: json.dumps(v, sort_keys=True)  # noqa: E731
    assert sorted(map(key, picked)) == sorted(map(key, bench.batch_views(bench.SEED)))


def test_image_error_statistics():
    a = np.zeros((4, 4, 4), np.uint8)
    b = a.copy()
    b[0, 0, 0] = 1
    b[1, 1, 2] = 3
    e = bench.image_error({0: a, 1: a}, {0: b, 1: a})
    assert e['views_compared'] == 2 and e['max_lsb'] == 3 and e['channels_over_1_lsb'] == 1
    assert abs(e["mean_lsb"] - 4 / 128) < 1e-9  # both views, 2 x 64 channels
