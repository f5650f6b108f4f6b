"""Benchmark of the transparent pass.

Default workload: the batched multi-view case -- 64 seeded sphere scenes at
square resolutions log-uniform in 256..2048 with 64..8192 spheres, Linked
List and Loop64 views with OIT_LAYERS 4..32 -- rendered as one batch with
RGBA8 records and an FP16 colour target (one CUDA graph, one persistent
resolve per view kind), against the plain path: one oit_render_frame per view
with RGBA32F records. One step = the whole batch of 64 frames. Metric:
transparent fragments (after early depth) per second in Mfragments/s;
ms_per_step is ms per batch. The line also carries the resolve alone (batched
vs one FP32 composite launch per view) with its HBM roofline.

Single-view workloads (--workload NAME): Loop64 / Spinlock at 1920x1080,
Linked List at 640x480, Interlock / Simple with 8x MSAA at 2560x1440, WBOIT at
3840x2160; one step = one frame.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl gb300|reference]

--impl reference times the CPU restatement of the reference's algorithm (the
oracle) on every host core: the reference itself is a Vulkan/GLSL program and
no graphics stack exists on either machine.
"""
import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (algorithm, width, height, layers, nodes/px, aa, spheres, rmin, rmax, percent transparent, alpha_min, alpha_width)
    'loop64_1920x1080_L16_1024spheres_60pct': ('loop64', 1920, 1080, 16, 8, 0, 1024, 0.03, 0.10, 60, 0.2, 0.6),
    'spinlock_1920x1080_L16_1024spheres_60pct': ('spinlock', 1920, 1080, 16, 8, 0, 1024, 0.03, 0.10, 60, 0.2, 0.6),
    'linkedlist_640x480_L8_256spheres': ('linkedlist', 640, 480, 8, 8, 0, 256, 0.05, 0.15, 100, 0.2, 0.6),
    'interlock_2560x1440_msaa8_L8_4096spheres': ('interlock', 2560, 1440, 8, 8, 4, 4096, 0.02, 0.08, 100, 0.2, 0.6),
    'simple_2560x1440_msaa8_L8_4096spheres': ('simple', 2560, 1440, 8, 8, 4, 4096, 0.02, 0.08, 100, 0.2, 0.6),
    'weighted_3840x2160_16384spheres': ('weighted', 3840, 2160, 8, 8, 0, 16384, 0.01, 0.05, 100, 0.05, 0.9),
    'linkedlist_1920x1080_L16_1024spheres': ('linkedlist', 1920, 1080, 16, 8, 0, 1024, 0.03, 0.10, 100, 0.2, 0.6),
    # the same frame with the COLOR pass in arrival order (OIT_FLAG_ARRIVAL_ORDER)
    'linkedlist_arrival_1920x1080_L16_1024spheres': ('linkedlist', 1920, 1080, 16, 8, 0, 1024, 0.03, 0.10, 100, 0.2,
                                                     0.6),
}
ARRIVAL_WORKLOADS = {'linkedlist_arrival_1920x1080_L16_1024spheres'}
ALGS = ['simple', 'linkedlist', 'loop', 'loop64', 'spinlock', 'interlock', 'weighted']
SEED = 2
BATCH_WORKLOAD = 'batch_64views_ll_loop64_mixed_vs_fp32'
DEFAULT_WORKLOAD = BATCH_WORKLOAD


def batch_views(seed=SEED, n=64):
    """The batched workload's views: square resolutions log-uniform in
    [256, 2048], sphere counts log-uniform in [64, 8192], radii 0.01-0.05,
    Linked List and Loop64 alternating, OIT_LAYERS cycling 4, 8, 16, 32 for
    each algorithm."""
    import numpy as np
    rng = np.random.default_rng(seed)
    views = []
    for k in range(n):
        side = int(round(256 * 8 ** rng.uniform()))
        spheres = int(round(64 * 128 ** rng.uniform()))
        alg = 'linkedlist' if k % 2 == 0 else 'loop64'
        L = [4, 8, 16, 32][(k // 2) % 4]
        views.append(dict(algorithm=alg, width=side, height=side, oit_layers=L, nodes_per_pixel=8, aa_type=0,
                          spheres=spheres, radius_min=0.01, radius_max=0.05, percent_transparent=100,
                          alpha_min=0.2, alpha_width=0.6, seed=seed * 1000 + k))
    return views


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--workload', default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS) + [BATCH_WORKLOAD])
    ap.add_argument('--views', type=int, default=64,
                    help='batch workload: the first N of its 64 views (smaller cases for profiling)')
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--raster-config', default='auto',
                    choices=['auto', 'per-view', 'per-view-longest-first', 'per-view-32', 'multi-view'],
                    help='batch workload: pin the tile-raster configuration instead of letting the graph capture '
                         'time the candidates (profilers distort those timings)')
    return ap.parse_args()


def workload_dict(name):
    if name == BATCH_WORKLOAD:
        vs = batch_views()
        return dict(workload=name, views=len(vs), algorithm='linkedlist+loop64', record_formats='rgba8 batched vs '
                    'rgba32f one view per call', resolutions='%d..%d square' % (min(v['width'] for v in vs),
                                                                                 max(v['width'] for v in vs)),
                    spheres='%d..%d' % (min(v['spheres'] for v in vs), max(v['spheres'] for v in vs)),
                    radius_min=0.01, radius_max=0.05, oit_layers='4,8,16,32', seed=SEED)
    alg, W, H, L, npp, aa, n, rmin, rmax, pct, amin, awid = WORKLOADS[name]
    return dict(workload=name, algorithm=alg, width=W, height=H, oit_layers=L, nodes_per_pixel=npp, aa_type=aa,
                spheres=n, radius_min=rmin, radius_max=rmax, percent_transparent=pct, alpha_min=amin,
                alpha_width=awid, seed=SEED)


def dtype_of(alg):
    return {'loop64': 'u64 keys + f32 blend', 'loop': 'u32 depth + f32 blend', 'weighted': 'f16 accum + f32'}.get(
        alg, 'u32 records + f32 blend')


# ---------------------------------------------------------------------------
# CPU leg (the oracle): a bounded sample of the same workload
# ---------------------------------------------------------------------------
def _oracle_frame(args):
    """(fragments, seconds[, RGBA8 image]) of one oracle frame of a workload;
    args = (workload, want_image[, oracle build: 'fp64' the FP64 oracle, or
    'fp32_omp' FP32 blending with OpenMP tile-parallel draws])."""
    wd, want_image = args[0], args[1]
    variant = args[2] if len(args) > 2 else 'fp64'
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as orc
    W, H = wd['width'], wd['height']
    # the oracle library's copy of the engine's scene generator (pinned to it
    # bit for bit by tests/test_oracle_workload.py): no product code here
    v, i, tpo = orc.make_scene(wd['spheres'], seed=wd['seed'], radius_min=wd['radius_min'],
                               radius_max=wd['radius_max'])
    sd = orc.make_camera(W, H)
    t = time.perf_counter()
    fr = orc.render(ALGS.index(wd['algorithm']), W, H, sd, v, i, tpo, wd['percent_transparent'],
                    oit_layers=wd['oit_layers'], nodes_per_pixel=wd['nodes_per_pixel'], aa_type=wd['aa_type'],
                    alpha_min=wd['alpha_min'], alpha_width=wd['alpha_width'], variant=variant)
    img, _ = fr.composite()
    dt = time.perf_counter() - t
    if want_image == 'image':
        return fr.fragment_count(), dt, img
    return fr.fragment_count(), dt


def cpu_baseline(wd, cores=1, frames=None, budget_s=15.0):
    """Oracle throughput on `cores` processes; each renders whole frames."""
    import oracle  # noqa: F401  (builds the oracle library if needed)
    ctx = mp.get_context('spawn')
    frames = frames or cores
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_oracle_frame, [(wd, 1)] * frames)
    wall = time.perf_counter() - t0
    frags = sum(r[0] for r in res)
    return frags, wall, res


def cpu_baseline_views(views, budget_s=15.0):
    """Oracle throughput (one process, one core) on whole frames of batch
    views, smallest first, until about budget_s of CPU work; also returns
    the oracle's images by view index."""
    import oracle  # noqa: F401
    ctx = mp.get_context('spawn')
    order = sorted(range(len(views)), key=lambda k: views[k]['width'] * views[k]['height'] + 1000 * views[k]['spheres'])
    frags, busy, n, images = 0, 0.0, 0, {}
    with ctx.Pool(1) as pool:
        for k, (f, dt, img) in zip(order, pool.imap(_oracle_frame, [(views[k], 'image') for k in order])):
            frags += f
            busy += dt
            n += 1
            images[k] = img
            if busy >= budget_s:
                break
        pool.terminate()
    return frags, busy, n, images


def oracle_images_all(views, procs=None):
    """The FP64 oracle's image of every view (a spawn pool, largest views
    first): the accuracy reference for the whole batch. Not timed."""
    import oracle  # noqa: F401  (builds the oracle library if needed)
    ctx = mp.get_context('spawn')
    procs = procs or max(1, min(len(views), os.cpu_count() or 1))
    order = sorted(range(len(views)), key=lambda k: -(views[k]['width'] * views[k]['height'] +
                                                       1000 * views[k]['spheres']))
    with ctx.Pool(procs) as pool:
        res = pool.map(_oracle_frame, [(views[k], 'image') for k in order], chunksize=1)
    return {k: r[2] for k, r in zip(order, res)}


def cpu_baseline_omp(works, budget_s=10.0):
    """The oracle's FP32 + OpenMP build (every host core, draws split over
    screen tiles) on whole frames of `works` in order until about budget_s;
    (fragments, seconds, frames, threads)."""
    import oracle  # noqa: F401  (builds both oracle libraries if needed)
    ctx = mp.get_context('spawn')
    frags, busy, n = 0, 0.0, 0
    with ctx.Pool(1) as pool:
        for f, dt in pool.imap(_oracle_frame, [(w, 1, 'fp32_omp') for w in works]):
            frags += f
            busy += dt
            n += 1
            if busy >= budget_s:
                break
        pool.terminate()
    return frags, busy, n, int(os.environ.get('OMP_NUM_THREADS', os.cpu_count() or 1))


def weighted_precision(wd, width=None, height=None):
    """The WBOIT precision study: the workload's scene (at its own size unless
    given) with FP16 and FP32 accumulators on the GPU against the FP64 oracle;
    per-pixel relative error of the accumulation (RGBA, where the oracle's
    magnitude is above 1e-3) and of the revealage. Not timed."""
    width = width or wd['width']
    height = height or wd['height']
    import importlib.util
    import numpy as np
    import vk_order_independent_transparency_gb300 as oit
    spec = importlib.util.spec_from_file_location('oit_parity_oracle', os.path.join(ROOT, 'oracle', 'oracle.py'))
    orc = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(orc)
    v, i, tpo = oit.make_scene(wd['spheres'], seed=wd['seed'], radius_min=wd['radius_min'], radius_max=wd['radius_max'])
    sd = oit.make_camera(width, height)
    fr = orc.render(orc.WEIGHTED, width, height, sd, v, i, tpo, wd['percent_transparent'],
                    alpha_min=wd['alpha_min'], alpha_width=wd['alpha_width'])
    acc_o = fr.buffer(orc.BUF_ACCUM, np.float64).reshape(-1, 4)
    rev_o = fr.buffer(orc.BUF_REVEAL, np.float64)
    mesh = oit.DeviceMesh(v, i)
    out = {'size': '%dx%d' % (width, height), 'reference': 'FP64 oracle'}
    for name, prec, dt in (('fp16', oit.OIT_WEIGHTED_FP16, np.float16), ('fp32', oit.OIT_WEIGHTED_FP32, np.float32)):
        with oit.Renderer(oit.make_state(oit.OIT_WEIGHTED, width, height, alpha_min=wd['alpha_min'],
                                         alpha_width=wd['alpha_width'], weighted_precision=prec)) as r:
            r.update_scene(sd)
            r.render_frame(mesh, tpo, wd['percent_transparent'])
            acc = r.read_buffer(oit.OIT_BUF_ACCUM, dt).astype(np.float64).reshape(-1, 4)
            rev = r.read_buffer(oit.OIT_BUF_REVEAL, dt).astype(np.float64)
        m = np.abs(acc_o) > 1e-3
        ra = np.abs(acc - acc_o)[m] / np.abs(acc_o)[m]
        rr = np.abs(rev - rev_o) / np.maximum(rev_o, 1e-3)
        out[name] = {'accum_rel_max': float(ra.max()), 'accum_rel_mean': float(ra.mean()),
                     'reveal_rel_max': float(rr.max()), 'reveal_rel_mean': float(rr.mean())}
    return out


def image_error(gpu_images, oracle_images, reference='FP64 oracle, same scenes'):
    """Max and mean absolute RGBA8 difference (LSB) over the views both have."""
    import numpy as np
    mx, tot, cnt, over = 0, 0.0, 0, 0
    for k, ref in oracle_images.items():
        d = np.abs(gpu_images[k].astype(np.int32) - ref.astype(np.int32))
        mx = max(mx, int(d.max()))
        tot += float(d.sum())
        cnt += d.size
        over += int((d > 1).sum())
    return {'views_compared': len(oracle_images), 'max_lsb': mx, 'mean_lsb': round(tot / max(cnt, 1), 6),
            'channels_over_1_lsb': over, 'reference': reference}


def reference_views():
    """The views the reference arm renders in one step of the batch workload:
    all 64 of the GPU arm's batch, largest first (so the pool's cores finish
    together)."""
    return sorted(batch_views(SEED), key=lambda vd: -(vd['width'] * vd['height'] + 1000 * vd['spheres']))


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi samples (every 20 ms) of SM clocks and throttle reasons.
    Started before the warm-up; mark() before and after the timed region
    delimits the samples that stop() summarises (if the region is shorter
    than one interval, the first sample after it began)."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.path = None

    def _rows(self):
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    parts = [p.strip() for p in line.split(',')]
                    if len(parts) >= 9 and line.endswith('\n'):
                        rows.append(parts)
        except OSError:
            pass
        return rows

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix='.csv')
            os.close(fd)
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.dev), '--query-gpu=' + self.Q,
                                          '--format=csv,noheader,nounits', '-lms', '20'],
                                         stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        t0 = time.time()
        while not self._rows() and time.time() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.01)

    def mark(self):
        return len(self._rows()) if self.proc else 0

    def stop(self, begin=0, end=None):
        if not self.proc:
            return None
        if end is not None and end <= begin:
            time.sleep(0.05)  # region shorter than one interval: take the next sample
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = self._rows()
        os.unlink(self.path)
        sel = rows[begin:end] if end is not None and end > begin else rows[begin:begin + 1]
        if not sel:
            return None
        sm = sorted(float(r[1]) for r in sel if r[1].replace('.', '').isdigit())
        mx = max((float(r[2]) for r in sel if r[2].replace('.', '').isdigit()), default=None)
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[k] for r in sel for k in range(4) if r[5 + k].lower().startswith('active')})
        return {'sm_mhz': sm[len(sm) // 2] if sm else None, 'sm_max_mhz': mx, 'reasons': reasons,
                'samples': len(sel), 'interval_ms': 20}


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------
def peaks():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


def ncu_traffic(kernel, workload):
    """dram bytes per launch from a committed ncu summary, if one exists."""
    path = os.path.join(ROOT, 'profiles', '%s_%s.txt' % (kernel, workload))
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.startswith('dram_bytes_per_launch:'):
                try:
                    return float(line.split(':', 1)[1].split()[0])
                except ValueError:
                    return None
    return None


def kernel_bytes(wd, r, frags, kept_entries, pairs_t, tris_t, color_bytes=16):
    """Algorithmic bytes per launch of the transparent raster (the A-buffer
    build) and of the composite, after the byte model of the pass: records
    written once and read once, aux words, the tail-blended colour target
    (16 B per pixel, 8 B with the FP16 colour target), the output, the opaque
    depth and colour the passes read. Returns (raster, composite,
    intermediate): `intermediate` is the pipeline's own traffic that the
    model does not count -- the raster's reads of the 96-byte setup records
    (+ 32 B perspective terms for WBOIT and the 8-byte bbox) once per
    triangle, and its 4-byte tile-list entries."""
    import vk_order_independent_transparency_gb300 as oit
    alg = wd['algorithm']
    msaa, _, ss = oit.aa_settings(wd['aa_type'])
    P = wd['width'] * wd['height'] * ss * ss
    S = msaa
    L = wd['oit_layers']
    opaque = wd['percent_transparent'] < 100
    # raster: opaque depth + colour in (with an opaque pass), colour target out
    rb = (S * P * 20 if opaque else 0) + P * color_bytes
    if alg == 'loop64':
        rb += P * L * 8  # every layer written (kept keys and the cleared ones)
    elif alg == 'loop':
        rb += P * L * 8  # depth and colour layers
    elif alg == 'linkedlist':
        rb += frags * 16 + P * 4  # nodes + heads
    elif alg in ('simple', 'spinlock', 'interlock'):
        rec = 16 if msaa > 1 else 8
        rb += kept_entries * rec + P * (4 if alg == 'simple' else 8)
    elif alg == 'weighted':
        rb += S * P * 10
    intermediate = tris_t * (96 + 8 + (32 if alg == 'weighted' else 0)) + pairs_t * 4
    # composite: A-buffer entries actually read + colour target + output
    out = wd['width'] * wd['height'] * 4
    if alg == 'loop64':
        cb = kept_entries * 8 + P * color_bytes + out
    elif alg == 'loop':
        cb = kept_entries * 8 + P * color_bytes + out
    elif alg == 'linkedlist':
        cb = frags * 16 + P * 4 + P * color_bytes + out
    elif alg == 'weighted':
        cb = S * P * (10 + (16 if opaque else 0)) + out
    else:
        rec = 16 if msaa > 1 else 8
        cb = kept_entries * rec + P * 4 + P * color_bytes + out
    return rb, cb, intermediate


def count_kept(wd, r):
    """A-buffer entries the composite reads (host readback, outside timing)."""
    import numpy as np
    import vk_order_independent_transparency_gb300 as oit
    alg = wd['algorithm']
    L = wd['oit_layers']
    msaa, _, ss = oit.aa_settings(wd['aa_type'])
    P = wd['width'] * wd['height'] * ss * ss
    if alg == 'loop64':
        ab = r.read_buffer(oit.OIT_BUF_ABUFFER).reshape(L, P, 2)
        n = (ab[:, :, 1] != 0xFFFFFFFF).sum(axis=0)
        return int(n.sum() + (n < L).sum())
    if alg == 'loop':
        ab = r.read_buffer(oit.OIT_BUF_ABUFFER).reshape(2 * L, P)
        n = (ab[:L] != 0xFFFFFFFF).sum(axis=0)
        return int(2 * n.sum() + (n < L).sum())
    if alg in ('simple', 'spinlock', 'interlock'):
        aux = r.read_buffer(oit.OIT_BUF_AUX)[:P]
        return int(np.minimum(aux, L).sum())
    return 0


class _DeviceArray:
    """A zero-copy view of an engine buffer for torch (__cuda_array_interface__)."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {'shape': shape, 'typestr': typestr, 'data': (ptr, False), 'version': 3}


def resolve_bytes(views, renderers, color_bytes=8):
    """Algorithmic bytes of one batched resolve: per pixel the colour target
    (8 B: FP16) in and RGBA8 (4 B) out; linked lists: the head (4 B) and every
    stored node (16 B); Loop64: every kept key plus the terminating empty key
    (8 B each); the work list (4 B per micro-tile, written and read) and the
    micro-tile lengths (read twice). Counted on the device, outside timing."""
    import torch
    import vk_order_independent_transparency_gb300 as oit
    total = 0
    tiles = 0
    for vd, r in zip(views, renderers):
        W, H, L = vd['width'], vd['height'], vd['oit_layers']
        P = W * H
        tiles += 8 * ((W + 15) // 16) * ((H + 15) // 16)  # work items: the micro-tiles of whole 16x16 tiles
        b = P * (color_bytes + 4)
        if vd['algorithm'] == 'linkedlist':
            b += P * 4 + 16 * min(r.fragment_count(), vd['nodes_per_pixel'] * P - 1)
        else:
            ptr, _ = r.buffer(oit.OIT_BUF_ABUFFER)
            keys = torch.as_tensor(_DeviceArray(ptr, (L, P), '<i8'), device='cuda')
            n = (keys != -1).sum(0)
            b += 8 * int(n.sum().item() + (n < L).sum().item())
        total += b
    return total + tiles * (4 + 4 + 2)


def run_gpu(a, wd, rank, world):
    import numpy as np
    import torch
    import vk_order_independent_transparency_gb300 as oit
    from vk_order_independent_transparency_gb300 import _build
    if rank == 0 or not os.path.exists(oit.LIB_PATH):
        _build.build()
    if world > 1:
        torch.distributed.barrier()
    dev = int(os.environ.get('LOCAL_RANK', '0'))
    torch.cuda.set_device(dev)
    alg = ALGS.index(wd['algorithm'])
    W, H = wd['width'], wd['height']
    v, i, tpo = oit.make_scene(wd['spheres'], seed=wd['seed'] + rank, radius_min=wd['radius_min'],
                               radius_max=wd['radius_max'])
    sd = oit.make_camera(W, H)
    flags = oit.OIT_FLAG_CUDA_GRAPH | (oit.OIT_FLAG_ARRIVAL_ORDER if wd['workload'] in ARRIVAL_WORKLOADS else 0)
    st = oit.make_state(alg, W, H, oit_layers=wd['oit_layers'], nodes_per_pixel=wd['nodes_per_pixel'],
                        aa_type=wd['aa_type'], alpha_min=wd['alpha_min'], alpha_width=wd['alpha_width'],
                        flags=flags)
    r = oit.Renderer(st)
    mesh = oit.DeviceMesh(v, i)
    r.update_scene(sd)
    stream = torch.cuda.current_stream().cuda_stream

    def step():
        r.render_frame(mesh, tpo, wd['percent_transparent'], None, stream)

    clocks = Clocks(dev)
    clocks.start()
    for _ in range(max(3, a.warmup)):
        step()
    torch.cuda.synchronize()
    frags = r.fragment_count()
    assert r.get_error() == 0

    # device-resident timing
    l0 = r.launch_count()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    m0 = clocks.mark()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(a.steps):
        step()
    ev1.record()
    torch.cuda.synchronize()
    elapsed_ms = ev0.elapsed_time(ev1)
    clk = clocks.stop(m0, clocks.mark())
    if world > 1:
        torch.distributed.barrier()
    launches = r.launch_count() - l0

    # per-pass timing (CUDA events on the launching stream), separate run
    r.profile_enable(True)
    for _ in range(a.steps):
        step()
    prof = r.profile_read()
    r.profile_enable(False)

    # end to end through the C ABI with host buffers (pinned), copies inside:
    # the scene as a template sphere and instance table (what a sphere scene
    # is), and as the flattened mesh the reference uploads
    def pinned(x):
        return torch.from_numpy(np.ascontiguousarray(x)).pin_memory().numpy()

    tv, ti, inst = (pinned(x) for x in oit.make_scene_instanced(
        wd['spheres'], seed=wd['seed'] + rank, radius_min=wd['radius_min'], radius_max=wd['radius_max']))
    vh, ih = pinned(v), pinned(i)
    oh = torch.empty((H, W, 4), dtype=torch.uint8).pin_memory().numpy()

    def e2e_time(frame):
        for _ in range(2):
            frame()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            frame()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    e2e_s = e2e_time(lambda: r.render_frame_instanced_host(tv, ti, inst, wd['percent_transparent'], oh, stream))
    e2e_flat_s = e2e_time(lambda: r.render_frame_host(vh, ih, tpo, wd['percent_transparent'], oh, stream))

    kept = count_kept(wd, r)
    tris_t = (i.shape[0] // tpo) * wd['percent_transparent'] // 100 * tpo
    res = dict(elapsed_ms=elapsed_ms, frags=frags, launches=launches, clocks=clk, prof=prof, e2e_s=e2e_s,
               h2d=int(tv.nbytes + ti.nbytes + inst.nbytes), d2h=int(oh.nbytes), kept=kept, tris_t=tris_t, r=r,
               e2e_flat_s=e2e_flat_s, h2d_flat=int(vh.nbytes + ih.nbytes))
    return res


def run_batch(a, rank):
    """Batched mixed-precision views (one CUDA graph, RGBA8 records) against the
    plain path (one oit_render_frame per view, RGBA32F records)."""
    import numpy as np
    import torch
    import vk_order_independent_transparency_gb300 as oit
    from vk_order_independent_transparency_gb300 import _build
    _build.build()
    torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', '0')))
    stream = torch.cuda.current_stream().cuda_stream
    vs = batch_views(SEED + rank)[:a.views]
    mixed, plain, meshes, host = [], [], [], []
    for vd in vs:
        v, i, tpo = oit.make_scene(vd['spheres'], seed=vd['seed'], radius_min=vd['radius_min'],
                                   radius_max=vd['radius_max'])
        sd = oit.make_camera(vd['width'], vd['height'])
        mesh = oit.DeviceMesh(v, i)
        meshes.append(mesh)
        host.append((v, i, tpo))
        for recs, fmt, flags in ((mixed, oit.OIT_RECORD_RGBA8, oit.OIT_FLAG_HALF_COLOR),
                                 (plain, oit.OIT_RECORD_RGBA32F, 0)):
            r = oit.Renderer(oit.make_state(ALGS.index(vd['algorithm']), vd['width'], vd['height'],
                                            oit_layers=vd['oit_layers'], nodes_per_pixel=vd['nodes_per_pixel'],
                                            alpha_min=vd['alpha_min'], alpha_width=vd['alpha_width'],
                                            record_format=fmt, flags=flags))
            r.update_scene(sd)
            recs.append(r)
    raster_pin = {'auto': None, 'per-view': {'multi_view': 0},
                  'per-view-longest-first': {'multi_view': 0, 'lane_order': 1},
                  'per-view-32': {'multi_view': 0, 'warps_per_sm': 32}, 'multi-view': {'multi_view': 1}}[a.raster_config]
    batch = oit.Batch(parallel_streams=16)
    batch.set_raster_config(raster_pin)
    batch.set_views([(r, m, h[2], 100) for r, m, h in zip(mixed, meshes, host)])

    def step_mixed():
        batch.render(stream)

    def step_plain():
        for r, m, h in zip(plain, meshes, host):
            r.render_frame(m, h[2], 100, None, stream)

    for _ in range(max(3, a.warmup)):
        step_mixed()
        step_plain()
    torch.cuda.synchronize()
    frags = sum(r.fragment_count() for r in mixed)
    frags_plain = sum(r.fragment_count() for r in plain)
    assert frags == frags_plain, (frags, frags_plain)
    for r in mixed + plain:
        assert r.get_error() == 0

    def timed(fn):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(a.steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    clocks = Clocks(int(os.environ.get('LOCAL_RANK', '0')))
    clocks.start()
    step_mixed()
    torch.cuda.synchronize()
    m0 = clocks.mark()
    torch.cuda.nvtx.range_push('batched_frames')
    t_mixed = timed(step_mixed)
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop(m0, clocks.mark())
    torch.cuda.nvtx.range_push('plain_frames')
    t_plain = timed(step_plain)
    torch.cuda.nvtx.range_pop()
    launches = batch.launch_count() * a.steps

    # A/B: the linked-list views' COLOR pass in arrival order (fragment-parallel,
    # HBM atomics, no tile binning) beside the same Loop64 views
    arrival = []
    for r, vd in zip(mixed, vs):
        if vd['algorithm'] != 'linkedlist':
            arrival.append(r)
            continue
        ra = oit.Renderer(oit.make_state(oit.OIT_LINKEDLIST, vd['width'], vd['height'], oit_layers=vd['oit_layers'],
                                         nodes_per_pixel=vd['nodes_per_pixel'], alpha_min=vd['alpha_min'],
                                         alpha_width=vd['alpha_width'],
                                         flags=oit.OIT_FLAG_HALF_COLOR | oit.OIT_FLAG_ARRIVAL_ORDER))
        ra.update_scene(oit.make_camera(vd['width'], vd['height']))
        arrival.append(ra)
    batch_arr = oit.Batch(parallel_streams=16)
    batch_arr.set_raster_config(raster_pin)
    batch_arr.set_views([(r, m, h[2], 100) for r, m, h in zip(arrival, meshes, host)])
    for _ in range(max(3, a.warmup)):
        batch_arr.render(stream)
    t_arrival = timed(lambda: batch_arr.render(stream))
    frags_arr = sum(r.fragment_count() for r in arrival)
    arr_err = max(r.get_error() for r in arrival)
    batch_arr.close()

    # per-pass times: every view rendered alone with section timing, and the
    # transparent raster's algorithmic bytes summed over the views
    sections = {}
    raster_bytes = 0
    raster_intermediate = 0
    for r, m, h, vd in zip(mixed, meshes, host, vs):
        r.profile_enable(True)
        r.render_frame(m, h[2], 100, None, stream)
        for k, (ms, n) in r.profile_read().items():
            if n:
                sections[k] = sections.get(k, 0.0) + ms / n
        r.profile_enable(False)
        vw = dict(vd, workload=BATCH_WORKLOAD)
        rb, _, ib = kernel_bytes(vw, r, r.fragment_count(), 0, 0, h[1].shape[0], color_bytes=8)
        raster_bytes += rb
        raster_intermediate += ib

    # end to end: every view's scene from pinned host memory, the batch, every
    # image back. The scene as template + instance table (what the sphere
    # scenes are), and as flattened meshes (what the reference uploads)
    outs = [torch.empty((vd['height'], vd['width'], 4), dtype=torch.uint8).pin_memory() for vd in vs]
    # instanced scenes: every view's spheres share one template (same stacks
    # and slices); the views' instance tables are packed in one buffer and
    # their images land in one buffer, so a step is one copy in and one out
    scenes = [oit.make_scene_instanced(vd['spheres'], seed=vd['seed'], radius_min=vd['radius_min'],
                                       radius_max=vd['radius_max']) for vd in vs]
    tv, ti = scenes[0][0], scenes[0][1]
    counts = [sc[2].shape[0] for sc in scenes]
    starts = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    # offsets in 4-byte words; the instance tables start 16-byte aligned
    inst_at = (tv.size + ti.size + 3) // 4 * 4
    scene_host = torch.zeros(inst_at + int(starts[-1]) * 8, dtype=torch.int32).pin_memory()
    scene_np = scene_host.numpy()
    scene_np[:tv.size] = tv.reshape(-1).view(np.int32)
    scene_np[tv.size:tv.size + ti.size] = ti.reshape(-1).view(np.int32)
    for sc, st in zip(scenes, starts[:-1]):
        scene_np[inst_at + 8 * st:inst_at + 8 * (st + sc[2].shape[0])] = sc[2].reshape(-1).view(np.int32)
    sizes = [vd['width'] * vd['height'] * 4 for vd in vs]
    out_at = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    # two sets (scene in, images out, a batch writing them), alternating by
    # step: a step's readback and the next step's upload run on copy streams
    # while the next batch renders
    pipe = []
    for _ in range(2):
        scene_dev = torch.empty_like(scene_host, device='cuda')
        scene_dev.copy_(scene_host)
        tv_dev = scene_dev[:tv.size].view(torch.float32).view(-1, 6)
        ti_dev = scene_dev[tv.size:tv.size + ti.size].view(-1, 3)
        inst_views = [oit.DeviceInstancedMesh.from_tensors(
            tv_dev, ti_dev, scene_dev[inst_at + 8 * st:inst_at + 8 * (st + n)].view(torch.float32).view(-1, 8))
            for st, n in zip(starts[:-1], counts)]
        out_dev = torch.empty(int(out_at[-1]), dtype=torch.uint8, device='cuda')
        out_host = torch.empty(int(out_at[-1]), dtype=torch.uint8).pin_memory()
        bt = oit.Batch(parallel_streams=16)
        bt.set_raster_config(raster_pin)
        bt.set_views([(r, m, 0, 100, out_dev.data_ptr() + int(o)) for r, m, o in zip(mixed, inst_views, out_at)])
        pipe.append(dict(scene=scene_dev, out=out_dev, host=out_host, batch=bt, meshes=inst_views,
                         uploaded=torch.cuda.Event(), rendered=torch.cuda.Event(), read=torch.cuda.Event()))
    up_stream, down_stream = torch.cuda.Stream(), torch.cuda.Stream()
    h2d, d2h = scene_host.nbytes, pipe[0]['host'].nbytes
    hv = [(torch.from_numpy(np.ascontiguousarray(v)).pin_memory(), torch.from_numpy(
        np.ascontiguousarray(i).view(np.int32)).pin_memory()) for v, i, _ in host]
    h2d_flat = sum(x.nbytes + y.nbytes for x, y in hv)

    def images_back():
        for r, o in zip(mixed, outs):
            ptr, nb = r.buffer(oit.OIT_BUF_OUTPUT)
            _copy_d2h(o, ptr, nb, stream)
        torch.cuda.current_stream().synchronize()

    e2e_k = [0]

    def step_e2e():
        x = pipe[e2e_k[0] % 2]
        e2e_k[0] += 1
        comp = torch.cuda.current_stream()
        with torch.cuda.stream(up_stream):
            up_stream.wait_event(x['rendered'])  # this set's previous batch has read its scene
            x['scene'].copy_(scene_host, non_blocking=True)
            x['uploaded'].record(up_stream)
        comp.wait_event(x['uploaded'])
        comp.wait_event(x['read'])  # this set's previous images are back on the host
        x['batch'].render(stream)
        x['rendered'].record(comp)
        with torch.cuda.stream(down_stream):
            down_stream.wait_event(x['rendered'])
            x['host'].copy_(x['out'], non_blocking=True)
            x['read'].record(down_stream)

    def e2e_drain():
        for st in (torch.cuda.current_stream(), up_stream, down_stream):
            st.synchronize()

    def step_e2e_flat():
        for (x, y), m in zip(hv, meshes):
            m.vertices.copy_(x, non_blocking=True)
            m.indices.copy_(y, non_blocking=True)
        batch.render(stream)
        images_back()

    def e2e_time(step, drain=None, warm=2):
        for _ in range(warm):
            step()
        if drain:
            drain()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            step()
        if drain:
            drain()  # every step's images are on the host before the clock stops
        return time.perf_counter() - t0

    e2e_s = e2e_time(step_e2e, e2e_drain, warm=6)  # each set's batch: plain frames, tuning, capture
    e2e_flat_s = e2e_time(step_e2e_flat)
    # the packed instanced steps' images are the flattened meshes' bit for bit
    e2e_same = all(torch.equal(x['host'][int(o0):int(o1)], o.reshape(-1))
                   for x in pipe for o, o0, o1 in zip(outs, out_at[:-1], out_at[1:]))

    # resolve alone: the batched persistent resolve of the mixed views against
    # one FP32-record composite launch per view, on the frames rendered above
    batch.render(stream)
    step_plain()

    def step_resolve_mixed():
        batch.resolve(stream)

    def step_resolve_plain():
        for r in plain:
            r.composite(None, stream)

    for _ in range(max(3, a.warmup)):
        step_resolve_mixed()
        step_resolve_plain()
    # NVTX ranges name the timed regions for profilers (ncu --nvtx-include)
    torch.cuda.nvtx.range_push('batched_resolve')
    t_res_mixed = timed(step_resolve_mixed)
    torch.cuda.nvtx.range_pop()
    torch.cuda.nvtx.range_push('plain_resolve')
    t_res_plain = timed(step_resolve_plain)
    torch.cuda.nvtx.range_pop()
    res_cfg = batch.resolve_config()
    raster_cfg = batch.raster_config()
    res_bytes = resolve_bytes(vs, mixed)
    batch.render(stream)
    images = [r.output() for r in mixed]
    # the FP64 verification resolve of every view's frame (not timed)
    fp64_images = {k: r.verify_composite_fp64(stream)[1] for k, r in enumerate(mixed)}
    return dict(frags=frags, t_mixed=t_mixed, t_plain=t_plain, launches=launches, clocks=clk, sections=sections,
                e2e_s=e2e_s, h2d=h2d, d2h=d2h, views=vs, t_res_mixed=t_res_mixed, t_res_plain=t_res_plain,
                res_cfg=res_cfg, res_bytes=res_bytes, e2e_flat_s=e2e_flat_s, h2d_flat=h2d_flat, e2e_same=e2e_same,
                raster_bytes=raster_bytes, raster_intermediate=raster_intermediate, images=images,
                fp64_images=fp64_images, raster_cfg=raster_cfg, t_arrival=t_arrival, frags_arr=frags_arr,
                arr_err=arr_err)


def _copy_d2h(host_tensor, dev_ptr, nbytes, stream):
    import ctypes
    import vk_order_independent_transparency_gb300 as oit
    rt = oit._cudart()
    rt.cudaMemcpyAsync.restype = ctypes.c_int
    rt.cudaMemcpyAsync(ctypes.c_void_p(host_tensor.data_ptr()), ctypes.c_void_p(dev_ptr), ctypes.c_size_t(nbytes), 2,
                       ctypes.c_void_p(stream))


def reduce_replicas(maxes, sums, world, device='cuda'):
    """The only exchange between replicas: the max over ranks of each timed
    duration and the sum over ranks of the work each rank did."""
    import torch
    m = torch.tensor([float(x) for x in maxes], dtype=torch.float64, device=device)
    s = torch.tensor([float(x) for x in sums], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(m, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(s)
    return m.tolist(), s.tolist()


def main_batch(a, rank, world):
    res = run_batch(a, rank)
    cpu_line = None
    cpu_omp_line = None
    accuracy = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        f, busy, n, _ = cpu_baseline_views(res['views'])
        cpu_line = {'value': round(f / busy / 1e6, 4), 'unit': 'Mfragments/s', 'cores': 1, 'kind': 'port',
                    'sample': '%d of the %d views (the smallest), whole frames, single-threaded FP64 oracle' % (
                        n, len(res['views']))}
        accuracy = image_error(res['images'], oracle_images_all(res['views']))
        accuracy['vs_fp64_gpu_resolve'] = image_error(
            res['images'], res['fp64_images'],
            'oit_verify_composite_fp64: the same frames resolved in FP64 on the GPU')
        order = sorted(range(len(res['views'])), key=lambda k: res['views'][k]['width'] * res['views'][k]['height'] +
                       1000 * res['views'][k]['spheres'])
        try:
            fo, bo, no, th = cpu_baseline_omp([res['views'][k] for k in order])
            cpu_omp_line = {'value': round(fo / bo / 1e6, 4), 'unit': 'Mfragments/s', 'cores': th, 'kind': 'port',
                            'sample': '%d of the %d views (the smallest), whole frames, the oracle built with FP32 '
                                      'blending and OpenMP tile-parallel draws' % (no, len(res['views']))}
        except Exception as e:  # the baseline build needs OpenMP
            cpu_omp_line = {'unavailable': str(e)[:200]}
    (t_mixed, t_plain, e2e_s, t_res_mixed, t_res_plain, e2e_flat_s), (total,) = reduce_replicas(
        [res['t_mixed'], res['t_plain'], res['e2e_s'], res['t_res_mixed'], res['t_res_plain'], res['e2e_flat_s']],
        [res['frags'] * a.steps], world)
    if rank != 0:
        return
    value = total / (t_mixed * 1e-3) / 1e6
    plain = total / (t_plain * 1e-3) / 1e6
    peak, peak_kind = peaks()
    sec = res['sections']
    resolve = resolve_line(res, a, world, total, t_res_mixed, t_res_plain, peak, peak_kind)
    line = {
        'metric': 'Mfragments/s', 'value': round(value, 3), 'unit': 'Mfragments/s', 'n_gpus': world,
        'steps': a.steps, 'warmup': a.warmup, 'ms_per_step': round(t_mixed / a.steps, 4), 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'rgba8 records, f16 colour target, f32 blend',
        'data': 'synthetic: 64 seeded UV-sphere scenes, inputs resident in HBM',
        'config': dict(workload_dict(BATCH_WORKLOAD), views=len(res['views']), fragments_per_batch=res['frags'],
                       parallelism='replicas' if world > 1 else 'single',
                       frame='all 64 views in one CUDA graph (views on 16 forked streams)',
                       l2='working set larger than L2, no flush'),
        'plain_fp32': {'value': round(plain, 3), 'unit': 'Mfragments/s', 'ms_per_step': round(t_plain / a.steps, 4),
                       'path': 'one oit_render_frame per view, RGBA32F records, no graph'},
        'speedup_vs_plain_fp32': round(value / plain, 3),
        'e2e': {'value': round(total / e2e_s / 1e6, 3), 'unit': 'Mfragments/s', 'h2d_bytes_per_step': res['h2d'],
                'd2h_bytes_per_step': res['d2h'], 'ms_per_step': round(e2e_s / a.steps * 1e3, 4),
                'path': 'oit_batch_render over instanced views: one template + the packed instance tables in, '
                        'the 64 RGBA8 images out (one copy each way per step); double-buffered, so a step\'s '
                        'readback and the next upload overlap the next batch',
                'images_equal_flat_mesh': bool(res['e2e_same'])},
        'e2e_flat_mesh': {'value': round(total / e2e_flat_s / 1e6, 3), 'unit': 'Mfragments/s',
                          'h2d_bytes_per_step': res['h2d_flat'], 'd2h_bytes_per_step': res['d2h'],
                          'ms_per_step': round(e2e_flat_s / a.steps * 1e3, 4),
                          'path': 'oit_batch_render over flattened meshes uploaded every step'},
        'roofline': resolve['roofline'],
        'raster_roofline': raster_roofline(res, sec, peak, peak_kind),
        'kernels': {k: {'ms_sum_over_views': round(v, 4)} for k, v in sec.items()},
        'arrival_order_ll': {'ms_per_step': round(res['t_arrival'] / a.steps, 4),
                             'value': round(res['frags_arr'] * a.steps / (res['t_arrival'] * 1e-3) / 1e6, 3),
                             'unit': 'Mfragments/s', 'fragments_equal': res['frags_arr'] == res['frags'],
                             'device_error_bits': int(res['arr_err']),
                             'path': 'the same batch with the linked-list views in OIT_FLAG_ARRIVAL_ORDER: '
                                     'fragment-parallel COLOR pass, warp-aggregated node counter, atomicExch '
                                     'heads in HBM, no tile binning; list order not deterministic'},
        'autotuned_raster': dict(res['raster_cfg'], picked_by='oit_batch_render timing the candidate graphs on the '
                                 'batch\'s frames (per-view launches at 36 and 32 warps per SM, views over the '
                                 'streams in view order or longest first, multi-view launches)'),
        'resolve': resolve,
        'cpu_baseline': cpu_line,
        'cpu_baseline_fp32_omp': cpu_omp_line,
        'accuracy': accuracy,
        'clocks': res['clocks'],
        'gpu_launches': int(res['launches']),
    }
    print(json.dumps(line))


def raster_roofline(res, sec, peak, peak_kind):
    """The batch's longest pass, the transparent raster (A-buffer build):
    the algorithmic bytes it writes and reads (records, aux words, the FP16
    colour target), summed over the 64 views, over its CUDA-event time summed
    over the views (each rendered alone). The setup-record reads, which the
    byte model does not count, are reported beside it."""
    ms = sec.get('transparent_raster', 0.0)
    gbs = res['raster_bytes'] / (ms * 1e-3) / 1e9 if ms else None
    return {'bound': 'issue/latency (integer edge tests, shading, per-pixel k-buffer steps)',
            'kernel': 'k_raster_transparent (summed over the 64 views)',
            'achieved': round(gbs, 1) if gbs else None, 'peak': peak, 'unit': 'GB/s',
            'frac': round(gbs / peak, 4) if gbs else None, 'traffic': None,
            'bytes_per_step': int(res['raster_bytes']), 'ms_per_step_summed': round(ms, 4),
            'intermediate_bytes': int(res['raster_intermediate']),
            'intermediate': 'setup records (96 B) and bboxes (8 B) read once per triangle; not algorithmic bytes',
            'peak_source': peak_kind}


def resolve_line(res, a, world, total, t_mixed, t_plain, peak, peak_kind):
    """The batched resolve (one persistent launch over every view, RGBA8
    records) against the plain path (one composite launch per view, FP32
    records): fragments of the batch resolved per second, and the batched
    kernel's achieved HBM bandwidth from its algorithmic bytes."""
    value = total / (t_mixed * 1e-3) / 1e6
    plain = total / (t_plain * 1e-3) / 1e6
    per = t_mixed / a.steps
    gbs = res['res_bytes'] / (per * 1e-3) / 1e9
    return {
        'value': round(value, 3), 'unit': 'Mfragments/s', 'ms_per_step': round(per, 4),
        'plain_fp32': {'value': round(plain, 3), 'unit': 'Mfragments/s', 'ms_per_step': round(t_plain / a.steps, 4),
                       'path': 'oit_composite per view, RGBA32F records'},
        'speedup_vs_plain_fp32': round(value / plain, 3),
        'roofline': {'bound': 'hbm', 'kernel': 'batched resolve: k_resolve_list + k_resolve_loop64 side by side '
                               '(+ work-list binning), per step', 'achieved': round(gbs, 1),
                     'peak': peak, 'unit': 'GB/s', 'frac': round(gbs / peak, 4),
                     'traffic': ncu_traffic('resolve', BATCH_WORKLOAD), 'bytes_per_step': int(res['res_bytes']),
                     'peak_source': peak_kind},
        'autotuned': res['res_cfg'],
    }


def main():
    a = parse()
    wd = workload_dict(a.workload)
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))

    if a.impl == 'reference':
        if rank != 0:
            return
        cores = os.cpu_count() or 1
        batch = a.workload == BATCH_WORKLOAD

        # the worker processes start (and load the oracle) once, before any timing
        pool = mp.get_context('spawn').Pool(cores)

        def ref_step(k):
            # one step = the workload: the batch's 64 views spread over the
            # cores (one whole frame per task), or one frame per core of a
            # single-view workload
            args = [(vd, 1) for vd in reference_views()] if batch else [(wd, 1)] * cores
            t0 = time.perf_counter()
            res = pool.map(_oracle_frame, args, chunksize=1)
            return sum(r[0] for r in res), time.perf_counter() - t0

        for k in range(max(1, min(a.warmup, 2))):
            ref_step(k)
        frags = 0
        wall = 0.0
        for k in range(a.steps):
            f, w = ref_step(k)
            frags += f
            wall += w
        pool.close()
        pool.join()
        value = frags / wall / 1e6
        line = {
            'impl': 'reference', 'metric': 'Mfragments/s', 'value': round(value, 4), 'unit': 'Mfragments/s',
            'n_gpus': a.gpus, 'steps': a.steps, 'warmup': a.warmup, 'ms_per_step': round(wall / a.steps * 1e3, 3),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64 blend',
            'data': 'synthetic: seeded UV-sphere scene', 'config': wd,
            'cpu_baseline': {'value': round(value, 4), 'unit': 'Mfragments/s', 'cores': cores, 'kind': 'port',
                             'sample': ('the whole 64-view batch per step, one view per task on %d processes' % cores)
                             if batch else '%d whole frames per step, one per core' % cores},
            'e2e': {'value': round(value, 4), 'unit': 'Mfragments/s', 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0},
            'note': 'reference Vulkan build unavailable on this box (no graphics stack); CPU restatement of the '
                    'reference shaders (oracle) timed instead',
        }
        print(json.dumps(line))
        return

    import torch
    if world > 1:
        torch.distributed.init_process_group('nccl' if torch.cuda.is_available() else 'gloo')
    if a.workload == BATCH_WORKLOAD:
        main_batch(a, rank, world)
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    res = run_gpu(a, wd, rank, world)
    (t_ms, e2e_s, e2e_flat_s), (frags_all,) = reduce_replicas([res['elapsed_ms'], res['e2e_s'], res['e2e_flat_s']],
                                                              [res['frags'] * a.steps], world)
    if rank != 0:
        torch.distributed.destroy_process_group()
        return
    value = frags_all / (t_ms * 1e-3) / 1e6
    e2e_value = frags_all / e2e_s / 1e6

    peak, peak_kind = peaks()
    prof = res['prof']
    rbytes, cbytes, ibytes = kernel_bytes(wd, res['r'], res['frags'], res['kept'], 0, res['tris_t'])
    kernels = {}
    for name, b in (('transparent_raster', rbytes), ('composite', cbytes)):
        ms, n = prof[name]
        if n:
            per = ms / n
            kernels[name] = {'ms': round(per, 4), 'bytes': int(b), 'gbs': round(b / (per * 1e-3) / 1e9, 1)}
            if name == 'transparent_raster':
                kernels[name]['intermediate_bytes'] = int(ibytes)
    for name in ('opaque_bin', 'opaque_raster', 'transparent_bin'):
        ms, n = prof[name]
        if n:
            kernels[name] = {'ms': round(ms / n, 4)}
    dom = max(kernels, key=lambda k: kernels[k]['ms'])
    droof = dom if 'gbs' in kernels[dom] else 'transparent_raster'
    k = kernels[droof]
    roofline = {'bound': 'hbm', 'kernel': droof, 'achieved': k['gbs'], 'peak': peak, 'unit': 'GB/s',
                'frac': round(k['gbs'] / peak, 4), 'traffic': ncu_traffic(droof, wd['workload']),
                'peak_source': peak_kind + ' (MEASURED_PEAKS.json hbm_gbs)' if peak_kind == 'measured' else peak_kind,
                'dominant_pass': dom}
    cpu = None
    cpu_omp = None
    precision = None
    if not a.no_cpu_baseline:
        try:
            fo, bo, no, th = cpu_baseline_omp([wd] * 5)
            cpu_omp = {'value': round(fo / bo / 1e6, 4), 'unit': 'Mfragments/s', 'cores': th, 'kind': 'port',
                       'sample': '%d whole frame(s) of the workload, the oracle built with FP32 blending and OpenMP '
                                 'tile-parallel draws' % no}
        except Exception as e:  # the baseline build needs OpenMP
            cpu_omp = {'unavailable': str(e)[:200]}
        f, w, runs = cpu_baseline(wd, cores=1, frames=1)
        n_more = max(0, min(4, int(12.0 / max(w, 1e-3)) - 1))
        if n_more:
            f2, w2, _ = cpu_baseline(wd, cores=1, frames=n_more)
            f += f2
            w += w2
        cpu = {'value': round(f / w / 1e6, 4), 'unit': 'Mfragments/s', 'cores': 1, 'kind': 'port',
               'sample': '%d whole frame(s) of the workload, single-threaded FP64 oracle' % (1 + n_more)}
        if wd['algorithm'] == 'weighted':
            precision = weighted_precision(wd)
    line = {
        'metric': 'Mfragments/s', 'value': round(value, 3), 'unit': 'Mfragments/s', 'n_gpus': world,
        'steps': a.steps, 'warmup': a.warmup, 'ms_per_step': round(t_ms / a.steps, 4), 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': dtype_of(wd['algorithm']),
        'data': 'synthetic: seeded UV-sphere scene (SplitMix64), inputs resident in HBM',
        'config': dict(wd, fragments_per_frame=res['frags'], parallelism='replicas' if world > 1 else 'single',
                       frame='one CUDA graph per frame (opaque + transparent binning, rasters, composite)',
                       l2='working set larger than L2 (A-buffer + triangle setup > 129 MB), no flush'),
        'e2e': {'value': round(e2e_value, 3), 'unit': 'Mfragments/s', 'h2d_bytes_per_step': res['h2d'],
                'd2h_bytes_per_step': res['d2h'], 'ms_per_step': round(e2e_s / a.steps * 1e3, 4),
                'path': 'oit_render_frame_instanced_host: template sphere + instance table in, RGBA8 out'},
        'e2e_flat_mesh': {'value': round(frags_all / e2e_flat_s / 1e6, 3), 'unit': 'Mfragments/s',
                          'h2d_bytes_per_step': res['h2d_flat'], 'd2h_bytes_per_step': res['d2h'],
                          'ms_per_step': round(e2e_flat_s / a.steps * 1e3, 4),
                          'path': 'oit_render_frame_host: flattened vertex + index buffers in, RGBA8 out'},
        'roofline': roofline,
        'kernels': kernels,
        'cpu_baseline': cpu,
        'cpu_baseline_fp32_omp': cpu_omp,
        'clocks': res['clocks'],
        'gpu_launches': int(res['launches']),
    }
    if precision:
        line['precision'] = precision
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()
