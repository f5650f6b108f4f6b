"""Shared helpers of the GPU parity tests: render one frame on the engine and
on the oracle from the same mesh and camera, and compare what the reference
defines bit for bit (fragment records, kept sets and their order) and what it
defines as colour (the RGBA8 image, within 1 LSB)."""
import numpy as np

import oracle as orc
import vk_order_independent_transparency_gb300 as oit

RECORD_WORDS = {oit.OIT_SIMPLE: None, oit.OIT_SPINLOCK: None, oit.OIT_INTERLOCK: None}


def scene(num_objects, width, height, seed=3, radius_min=0.05, radius_max=0.15, half_extent=1.0):
    v, i, tpo = oit.make_scene(num_objects, seed=seed, radius_min=radius_min, radius_max=radius_max,
                               half_extent=half_extent)
    return v, i, tpo, oit.make_camera(width, height)


def render_gpu(algorithm, width, height, v, i, tpo, sd, percent=100, **kw):
    st = oit.make_state(algorithm, width, height, **kw)
    r = oit.Renderer(st)
    mesh = oit.DeviceMesh(v, i)
    r.update_scene(sd)
    r.render_frame(mesh, tpo, percent)
    res = collect(r, algorithm, **kw)
    res['mesh'] = mesh
    return res


def collect(r, algorithm, **kw):
    """The frame state of a Renderer after a frame: image, A-buffer, aux
    words, colour target, depth, fragment count, error bits (and the WBOIT
    accumulators)."""
    res = {
        'image': r.output(),
        'abuf': r.read_buffer(oit.OIT_BUF_ABUFFER),
        'aux': r.read_buffer(oit.OIT_BUF_AUX),
        'auxdepth': r.read_buffer(oit.OIT_BUF_AUXDEPTH),
        'counter': r.read_buffer(oit.OIT_BUF_COUNTER),
        'color': (r.read_buffer(oit.OIT_BUF_COLOR, np.float16).astype(np.float32)
                  if kw.get('flags', 0) & oit.OIT_FLAG_HALF_COLOR else
                  r.read_buffer(oit.OIT_BUF_COLOR, np.float32)).reshape(-1, 4),
        'depth': r.read_buffer(oit.OIT_BUF_DEPTH),
        'fragments': r.fragment_count(),
        'error': r.get_error(),
        'renderer': r,
    }
    if algorithm == oit.OIT_WEIGHTED:
        if kw.get('weighted_precision', 0) == oit.OIT_WEIGHTED_FP32:
            res['accum'] = r.read_buffer(oit.OIT_BUF_ACCUM, np.float32).reshape(-1, 4).astype(np.float64)
            res['reveal'] = r.read_buffer(oit.OIT_BUF_REVEAL, np.float32).astype(np.float64)
        else:
            res['accum'] = r.read_buffer(oit.OIT_BUF_ACCUM, np.float16).reshape(-1, 4).astype(np.float64)
            res['reveal'] = r.read_buffer(oit.OIT_BUF_REVEAL, np.float16).astype(np.float64)
    return res


def render_oracle(algorithm, width, height, v, i, tpo, sd, percent=100, oit_layers=8, nodes_per_pixel=8,
                  aa_type=0, tail_blend=True, alpha_min=0.2, alpha_width=0.6, record_format=0, **_):
    fr = orc.render(algorithm, width, height, sd, v, i, tpo, percent, oit_layers=oit_layers,
                    nodes_per_pixel=nodes_per_pixel, aa_type=aa_type, tail_blend=tail_blend, alpha_min=alpha_min,
                    alpha_width=alpha_width, record_fp32=record_format == oit.OIT_RECORD_RGBA32F)
    state = {
        'abuf': fr.buffer(orc.BUF_ABUFFER),
        'aux': fr.buffer(orc.BUF_AUX),
        'auxdepth': fr.buffer(orc.BUF_AUXDEPTH),
        'counter': fr.buffer(orc.BUF_COUNTER),
        'depth': fr.buffer(orc.BUF_DEPTH),
        'color_samples': fr.buffer(orc.BUF_COLOR, np.float64).reshape(fr.msaa, -1, 4),
        'accum': fr.buffer(orc.BUF_ACCUM, np.float64).reshape(-1, 4),
        'reveal': fr.buffer(orc.BUF_REVEAL, np.float64),
        'fragments': fr.fragment_count(),
    }
    out8, lin = fr.composite()
    state['image'] = out8
    state['linear'] = lin
    state['frame'] = fr
    return state


def walk_lists(pool_words, heads, fp32=False):
    """Each list's entries in list order: (colour, depth, mask) per node; with
    RGBA32F nodes the colour is the four float bit patterns."""
    pool = pool_words.reshape(-1, 8 if fp32 else 4)
    out = []
    for h in heads:
        seq = []
        off = int(h)
        guard = 0
        while off:
            n = pool[off]
            if fp32:
                seq.append((tuple(int(x) for x in n[:4]), int(n[4]), int(n[5])))
                off = int(n[6])
            else:
                seq.append((int(n[0]), int(n[1]), int(n[2])))
                off = int(n[3])
            guard += 1
            assert guard <= pool.shape[0], 'cycle in linked list'
        out.append(seq)
    return out


def compare_abuffer(algorithm, g, o, L, P, coverage, ssn=1, fp32=False):
    """Bit-exact comparison of the algorithm's A-buffer state. With sample
    shading (ssn > 1) every sample has its own A-buffer block."""
    if algorithm in (oit.OIT_SIMPLE, oit.OIT_SPINLOCK, oit.OIT_INTERLOCK):
        np.testing.assert_array_equal(g['aux'][:ssn * P], o['aux'][:ssn * P])
        words = 4 if coverage else 2
        ga = g['abuf'][:ssn * L * P * words].reshape(ssn, L, P, words)
        oa = o['abuf'][:ssn * L * P * words].reshape(ssn, L, P, words)
        n = np.minimum(o['aux'][:ssn * P].reshape(ssn, P), L)
        for s in range(ssn):
            for layer in range(L):
                sel = n[s] > layer
                np.testing.assert_array_equal(ga[s, layer][sel], oa[s, layer][sel], err_msg='sample %d layer %d' % (s, layer))
        if algorithm != oit.OIT_SIMPLE:
            np.testing.assert_array_equal(g['auxdepth'][:ssn * P], o['auxdepth'][:ssn * P])
    elif algorithm == oit.OIT_LINKEDLIST:
        assert g['counter'][0] == o['counter'][0]
        assert walk_lists(g['abuf'], g['aux'][:ssn * P], fp32) == walk_lists(o['abuf'], o['aux'][:ssn * P], fp32)
    elif algorithm == oit.OIT_LOOP:
        ga = g['abuf'][:ssn * 2 * L * P].reshape(ssn, 2 * L, P)
        oa = o['abuf'][:ssn * 2 * L * P].reshape(ssn, 2 * L, P)
        np.testing.assert_array_equal(ga[:, :L], oa[:, :L])
        for s in range(ssn):
            count = (oa[s, :L] != 0xFFFFFFFF).sum(axis=0)
            for layer in range(L):
                sel = count > layer
                np.testing.assert_array_equal(ga[s, L + layer][sel], oa[s, L + layer][sel])
    elif algorithm == oit.OIT_LOOP64:
        np.testing.assert_array_equal(g['abuf'][:ssn * 2 * L * P], o['abuf'][:ssn * 2 * L * P])
        if fp32:
            keys = o['abuf'][:ssn * 2 * L * P].reshape(-1, 2)
            used = keys[:, 1] != 0xFFFFFFFF
            base = ssn * 2 * L * P
            gp = g['abuf'][base:base + 4 * ssn * L * P].reshape(-1, 4)
            op = o['abuf'][base:base + 4 * ssn * L * P].reshape(-1, 4)
            np.testing.assert_array_equal(gp[used], op[used])


def check_pair(alg, g, o, W, H, L, aa=0, ss=1, fp32=False, color_atol=2e-5, color_rtol=0.0):
    """Every bit-exact and colour comparison of one engine frame against the
    oracle's: error bits, fragment counts, A-buffer state, the tail-blended
    colour target (2e-5 absolute) and the RGBA8 image (1 LSB)."""
    msaa, sample_shading, _ = oit.aa_settings(aa)
    coverage = msaa > 1 and not sample_shading
    ssn = msaa if sample_shading else 1
    P = W * H * ss * ss
    assert g['error'] == 0
    assert g['fragments'] == o['fragments']
    if alg != oit.OIT_WEIGHTED:
        compare_abuffer(alg, g, o, L, P, coverage, ssn, fp32)
        if ssn > 1:
            ref_col = o['color_samples'].reshape(-1, 4)
        else:
            ref_col = o['color_samples'].mean(axis=0)
        np.testing.assert_allclose(g['color'][:ssn * P], ref_col, atol=color_atol, rtol=color_rtol)
    return compare_images(g, o)


def compare_images(g, o, max_lsb=1):
    d = np.abs(g['image'].astype(np.int32) - o['image'].astype(np.int32))
    assert d.max() <= max_lsb, 'image differs by %d LSB at %s' % (d.max(), np.argwhere(d == d.max())[:4])
    return int(d.max()), float((d > 0).mean())
