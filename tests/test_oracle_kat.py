"""Known-answer tests of the CPU oracle: the README traces of the reference.

Each trace (README.md:45, 53-66, 72, 80, 86-96) uses OIT_LAYERS=2 and four
fragments (c4, 0.4), (c2, 0.2), (c1, 0.1), (c3, 0.3); these tests inject the
fragments in the trace's arrival order and check the stored A-buffer, which
fragments were tail blended (and in which order) and the final colour.
"""
import numpy as np
import pytest

import oracle as orc

C = {1: (0.80, 0.10, 0.10, 0.50), 2: (0.10, 0.70, 0.20, 0.40), 3: (0.20, 0.30, 0.90, 0.60),
     4: (0.60, 0.60, 0.05, 0.30)}
Z = {1: 0.1, 2: 0.2, 3: 0.3, 4: 0.4}
BG = np.array([0.2, 0.2, 0.2, 0.2], np.float32).astype(np.float64)


def f32(x):
    return float(np.float32(x))


def packed(k, L):
    c = C[k]
    r, g, b = (L.or_srgb_encode(f32(v)) for v in c[:3])
    a = int(np.rint(np.float32(c[3]) * np.float32(255.0)))
    return r | (g << 8) | (b << 16) | (a << 24)


def dec_premult(p, L):
    a = ((p >> 24) & 255) / 255.0
    return np.array([L.or_srgb_decode(p & 255) * a, L.or_srgb_decode((p >> 8) & 255) * a,
                     L.or_srgb_decode((p >> 16) & 255) * a, a])


def own_premult(k):
    c = [f32(v) for v in C[k]]
    return np.array([c[0] * c[3], c[1] * c[3], c[2] * c[3], c[3]])


def over(top, bottom):
    return top + (1.0 - top[3]) * bottom


def rop(dst, src):  # hardware blend: src over dst
    return src + (1.0 - src[3]) * dst


def inject(fr, seq, pixel_of=None):
    xy = [(pixel_of[i] if pixel_of else 0, 0) for i in range(len(seq))]
    fr.inject(xy, [C[k] for k in seq], [Z[k] for k in seq])


def final(fr):
    out8, lin = fr.composite()
    return lin[0, 0], out8[0, 0]


def test_simple_first_k(oracle_lib):
    """README.md:45: Simple stores the first two fragments and tail blends the rest."""
    L = oracle_lib.lib()
    fr = orc.Frame(orc.SIMPLE, 1, 1, oit_layers=2)
    inject(fr, [4, 2, 1, 3])
    ab = fr.buffer(orc.BUF_ABUFFER).reshape(2, 2)
    assert list(ab[:, 1].view(np.float32)) == [np.float32(0.4), np.float32(0.2)]
    assert list(ab[:, 0]) == [packed(4, L), packed(2, L)]
    assert fr.buffer(orc.BUF_AUX)[0] == 4
    tail = rop(rop(BG, own_premult(1)), own_premult(3))
    expect = over(over(dec_premult(packed(2, L), L), dec_premult(packed(4, L), L)), tail)
    lin, _ = final(fr)
    np.testing.assert_allclose(lin, expect, rtol=0, atol=1e-12)


def test_linked_list_pool(oracle_lib):
    """README.md:53-66: a 4-element pool, two pixels, (c3, 0.3) tail blended."""
    L = oracle_lib.lib()
    fr = orc.Frame(orc.LINKEDLIST, 2, 1, oit_layers=2, nodes_per_pixel=2)  # pool = 2*2 = 4 nodes
    seq = [4, 1, 2, 3]
    px = [0, 1, 0, 0]
    fr.inject([(p, 0) for p in px], [C[k] for k in seq], [Z[k] for k in seq])
    pool = fr.buffer(orc.BUF_ABUFFER).reshape(4, 4)
    assert list(pool[1]) == [packed(4, L), np.float32(0.4).view(np.uint32), 0, 0]
    assert list(pool[2]) == [packed(1, L), np.float32(0.1).view(np.uint32), 0, 0]
    assert list(pool[3]) == [packed(2, L), np.float32(0.2).view(np.uint32), 0, 1]
    assert list(fr.buffer(orc.BUF_AUX)) == [3, 2]
    assert fr.buffer(orc.BUF_COUNTER)[0] == 4  # the counter also counts the overflowed fragment
    out8, lin = fr.composite()
    p1 = rop(rop(BG, own_premult(3)), over(dec_premult(packed(2, L), L), dec_premult(packed(4, L), L)))
    p2 = rop(BG, dec_premult(packed(1, L), L))
    np.testing.assert_allclose(lin[0, 0], p1, atol=1e-12)
    np.testing.assert_allclose(lin[0, 1], p2, atol=1e-12)


def test_linked_list_composite_tail(oracle_lib):
    """Lists longer than OIT_LAYERS: the nearest L are sorted, the rest tail blended in list order."""
    L = oracle_lib.lib()
    fr = orc.Frame(orc.LINKEDLIST, 1, 1, oit_layers=2, nodes_per_pixel=8)
    inject(fr, [4, 2, 1, 3])
    # list order (head first) is reverse arrival: 3, 1, 2, 4
    # gather (3, 1) -> sorted (1, 3); then 2: evicts 3; then 4: evicted itself
    tail = over(dec_premult(packed(3, L), L), dec_premult(packed(4, L), L))
    front = over(dec_premult(packed(1, L), L), dec_premult(packed(2, L), L))
    lin, _ = final(fr)
    np.testing.assert_allclose(lin, rop(BG, over(front, tail)), atol=1e-12)


def test_loop32(oracle_lib):
    """README.md:72: depths (0.1, 0.2) kept, (c4, 0.4) and (c3, 0.3) tail blended."""
    L = oracle_lib.lib()
    fr = orc.Frame(orc.LOOP, 1, 1, oit_layers=2)
    inject(fr, [4, 2, 1, 3])
    ab = fr.buffer(orc.BUF_ABUFFER)
    assert list(ab[:2].view(np.float32)) == [np.float32(0.1), np.float32(0.2)]
    assert list(ab[2:]) == [packed(1, L), packed(2, L)]
    tail = rop(rop(BG, own_premult(4)), own_premult(3))
    lin, _ = final(fr)
    np.testing.assert_allclose(lin, rop(tail, over(dec_premult(packed(1, L), L), dec_premult(packed(2, L), L))),
                               atol=1e-12)


def test_loop32_dedups_equal_depths(oracle_lib):
    """oitLoop.frag.glsl:87-92: equal depths share one slot; the colour is the last writer's."""
    L = oracle_lib.lib()
    fr = orc.Frame(orc.LOOP, 1, 1, oit_layers=4)
    fr.inject([(0, 0)] * 3, [C[1], C[2], C[3]], [0.5, 0.5, 0.25])
    ab = fr.buffer(orc.BUF_ABUFFER)
    assert list(ab[:4].view(np.float32)[:2]) == [np.float32(0.25), np.float32(0.5)]
    assert ab[2] == 0xFFFFFFFF and ab[3] == 0xFFFFFFFF
    assert ab[4] == packed(3, L) and ab[5] == packed(2, L)


def test_loop64(oracle_lib):
    """README.md:80: ((c1,0.1),(c2,0.2)) kept; c4 then c3 tail blended (decoded from rgba8)."""
    L = oracle_lib.lib()
    fr = orc.Frame(orc.LOOP64, 1, 1, oit_layers=2)
    inject(fr, [4, 2, 1, 3])
    ab = fr.buffer(orc.BUF_ABUFFER).view(np.uint64)
    k = lambda i: (int(np.float32(Z[i]).view(np.uint32)) << 32) | packed(i, L)
    assert [int(x) for x in ab] == [k(1), k(2)]
    tail = rop(rop(BG, dec_premult(packed(4, L), L)), dec_premult(packed(3, L), L))
    lin, _ = final(fr)
    np.testing.assert_allclose(lin, rop(tail, over(dec_premult(packed(1, L), L), dec_premult(packed(2, L), L))),
                               atol=1e-12)


@pytest.mark.parametrize('alg', [orc.SPINLOCK, orc.INTERLOCK])
def test_spinlock_trace(oracle_lib, alg):
    """README.md:86-96: critical-section order c3, c2, c4, c1; c4 and c3 end up tail blended."""
    L = oracle_lib.lib()
    fr = orc.Frame(alg, 1, 1, oit_layers=2)
    inject(fr, [3, 2, 4, 1])
    ab = fr.buffer(orc.BUF_ABUFFER).reshape(2, 2)
    assert list(ab[:, 0]) == [packed(1, L), packed(2, L)]
    assert fr.buffer(orc.BUF_AUXDEPTH)[0] == np.float32(0.3).view(np.uint32)
    assert fr.buffer(orc.BUF_AUX)[0] == 4
    tail = rop(rop(BG, own_premult(4)), dec_premult(packed(3, L), L))
    lin, _ = final(fr)
    np.testing.assert_allclose(lin, rop(tail, over(dec_premult(packed(1, L), L), dec_premult(packed(2, L), L))),
                               atol=1e-12)


def test_no_tail_blend_drops_overflow(oracle_lib):
    L = oracle_lib.lib()
    fr = orc.Frame(orc.SIMPLE, 1, 1, oit_layers=2, tail_blend=False)
    inject(fr, [4, 2, 1, 3])
    lin, _ = final(fr)
    expect = rop(BG, over(dec_premult(packed(2, L), L), dec_premult(packed(4, L), L)))
    np.testing.assert_allclose(lin, expect, atol=1e-12)


def test_bubble_sort_equal_depths(oracle_lib):
    """bubbleSort swaps on >= (oitCompositeDefines.glsl:51-89): equal depths are reordered."""
    L = oracle_lib.lib()
    fr = orc.Frame(orc.SIMPLE, 1, 1, oit_layers=4)
    fr.inject([(0, 0)] * 3, [C[1], C[2], C[3]], [0.5, 0.5, 0.5])
    lin, _ = final(fr)
    # n = 3: i=1: j=0 swap (1,2)->(2,1,3); j=1 swap -> (2,3,1); i=0: j=0 swap -> (3,2,1)
    d = lambda k: dec_premult(packed(k, L), L)
    np.testing.assert_allclose(lin, rop(BG, over(over(d(3), d(2)), d(1))), atol=1e-12)


def test_weighted_blended(oracle_lib):
    """oitWeighted.frag.glsl:53-79 and 98-108 in FP64."""
    fr = orc.Frame(orc.WEIGHTED, 1, 1)
    seq = [1, 2, 3]
    vz = [-2.0, -3.0, -4.5]
    fr.inject([(0, 0)] * 3, [C[k] for k in seq], [Z[k] for k in seq], view_z=vz)
    acc = np.zeros(4)
    rev = 1.0
    for k, z in zip(seq, vz):
        c = own_premult(k)
        dz = -np.float32(z) * 10.0
        dw = min(max(0.03 / (1e-5 + (dz / 200.0) ** 4), 1e-2), 3e3)
        aw = min(1.0, max(c) * 40.0 + 0.01) ** 2
        acc += c * aw * dw
        rev *= 1.0 - c[3]
    lin, _ = final(fr)
    rgb = acc[:3] / max(acc[3], 1e-5) * (1 - rev) + BG[:3] * rev
    a = rev * (1 - rev) + BG[3] * rev
    np.testing.assert_allclose(lin, list(rgb) + [a], atol=1e-12)


def test_coverage_resolve(oracle_lib):
    """MSAA coverage shading: per-sample blends of masked fragments, averaged (oitSimple.frag.glsl:142-159)."""
    L = oracle_lib.lib()
    fr = orc.Frame(orc.SIMPLE, 1, 1, oit_layers=4, aa_type=1)  # 4x MSAA
    fr.inject([(0, 0)] * 2, [C[1], C[2]], [0.1, 0.2], mask=[0b0011, 0b0110])
    lin, _ = final(fr)
    d = lambda k: dec_premult(packed(k, L), L)
    samples = [d(1), over(d(1), d(2)), d(2), np.zeros(4)]
    col_sum = sum(samples) / 4.0
    np.testing.assert_allclose(lin, rop(BG, col_sum), atol=1e-12)


def test_srgb_encode_is_exact(oracle_lib):
    L = oracle_lib.lib()
    thr = [L.or_srgb_threshold(k) for k in range(255)]
    assert all(a < b for a, b in zip(thr, thr[1:]))
    for k in range(255):
        t = np.float32(thr[k])
        below = np.nextafter(t, np.float32(0))
        assert L.or_srgb_encode(float(t)) == k + 1
        assert L.or_srgb_encode(float(below)) == k
    assert L.or_srgb_encode(0.0) == 0 and L.or_srgb_encode(1.0) == 255
    assert L.or_srgb_encode(float('nan')) == 0


def test_oracle_clips_at_the_near_plane(oracle_lib):
    """A triangle with one vertex behind the near plane is drawn in part (the
    part in front of the plane; fragments with window depth down to 0), one
    wholly behind it is not drawn."""
    import numpy as np
    import vk_order_independent_transparency_gb300 as oit
    W, H = 64, 48
    sd = oit.make_camera(W, H, eye=(0.0, 0.0, 0.0), target=(0.0, 0.0, -1.0), z_near=0.5, z_far=10.0)
    # a large triangle in the y = 0 plane reaching from 2 units in front to 0.2 (closer than near)
    def tri(zs):
        v = np.zeros((3, 10), np.float32)
        v[:, 0] = [-1.0, 1.0, 0.0]
        v[:, 1] = [-0.3, -0.3, 0.3]
        v[:, 2] = zs
        v[:, 4] = 1.0
        v[:, 6:10] = [0.8, 0.4, 0.2, 1.0]
        return v
    idx = np.array([[0, 1, 2]], np.uint32)
    fr = oracle_lib.render(oracle_lib.LINKEDLIST, W, H, sd, tri([-2.0, -2.0, -0.2]), idx, 1, 100, oit_layers=4)
    n_cut = fr.fragment_count()
    assert n_cut > 0
    ab = fr.buffer(oracle_lib.BUF_ABUFFER).reshape(-1, 4)
    depths = ab[1:n_cut + 1, 1].view(np.float32)
    assert depths.min() < 0.05  # fragments reach the near plane
    fr2 = oracle_lib.render(oracle_lib.LINKEDLIST, W, H, sd, tri([-0.3, -0.2, -0.1]), idx, 1, 100, oit_layers=4)
    assert fr2.fragment_count() == 0
