// C++ host engine behind the C ABI (include/oit_gb300.h).
//
// oit_context plays the role of the reference's Sample (oit.h:165-426): it
// owns the per-frame buffers sized by the algorithm (createFrameImages,
// oit.cpp:45-220), records the transparent pass on a CUDA stream
// (clearTransparent* / drawTransparent*, oitRender.cpp:156-425) and resolves
// to the back buffer (copyOffscreenToBackBuffer, main.cpp:645-774). Every
// entry point returns a status and never aborts.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "../../include/oit_gb300.h"
#include "oit_internal.h"

// defined with the C entry points below
extern "C" {
static oit::MeshRef view_mesh(const oit_view_frame& v);
static uint32_t view_tpo(const oit_view_frame& v);
}

namespace {

// Test aid (oit_debug_fail_allocations): the device allocation this many
// allocations from now fails once, as an exhausted cudaMalloc would; -1: off.
std::atomic<int> g_fail_alloc_countdown{-1};

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    if (n == 0) n = 16;
    int c = g_fail_alloc_countdown.load();
    while (c >= 0 && !g_fail_alloc_countdown.compare_exchange_weak(c, c - 1)) {
    }
    if (c == 0) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    bytes = n;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

bool debug_enabled() {
  static int v = -1;
  if (v < 0) v = std::getenv("OIT_DEBUG") ? 1 : 0;
  return v == 1;
}

int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return OIT_OK;
  if (debug_enabled()) std::fprintf(stderr, "oit: CUDA error in %s: %s\n", where, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return OIT_ERR_OUT_OF_MEMORY;
  return OIT_ERR_CUDA;
}

#define OIT_TRY_CUDA(expr, where)                   \
  do {                                              \
    cudaError_t _e = (expr);                        \
    if (_e != cudaSuccess) return cuda_status(_e, where); \
  } while (0)

}  // namespace

struct oit_context {
  oit_state st{};
  int msaa = 1, sample_shading = 0, supersample = 1;
  int W = 0, H = 0, RW = 0, RH = 0;
  uint32_t P = 0;
  int S = 1, coverage = 0, L = 1;
  int ssn = 1;  // samples with their own A-buffer (sample shading); WBOIT never uses them
  int tiles_x = 0, tiles_y = 0, num_tiles = 0, key_bits = 1;
  uint32_t capacity = 0;
  bool has_scene = false;

  // Scene constants (SceneData): oit_update_scene writes them into the next
  // slot of a pinned host ring; the next frame call copies the newest slot
  // into scene_dev on its stream before any kernel reads it, so a captured
  // graph reads the camera of the frame it renders. A slot is rewritten only
  // after the copy that last read it has run (its event).
  static constexpr int kSceneSlots = 4;
  static constexpr size_t kSceneBytes = 32 * sizeof(float);
  float* scene_ring = nullptr;  // pinned, kSceneSlots x 32 floats
  cudaEvent_t scene_ev[kSceneSlots] = {};
  bool scene_ev_used[kSceneSlots] = {};
  int scene_slot = 0;
  bool scene_dirty = false;
  float4 background = make_float4(0.2f, 0.2f, 0.2f, 0.2f);

  DevBuf depth, opaque_color, color, abuf, aux, auxdepth, counter, accum, reveal, out, out_linear, err, frag;
  DevBuf bbox, setup, persp, pair_count, pair_offset, scan_tmp, total;
  DevBuf keys, tris, keys_alt, tris_alt, hist, tile_begin, tile_end;
  DevBuf mesh_v, mesh_i;
  DevBuf scene_dev;  // proj_view then view, read by k_setup
  DevBuf lens;  // per 8x4 micro-tile fragment counts for the batched resolve
  size_t tri_cap = 0, pair_cap = 0;
  uint32_t bin_tris = 0, bin_opaque_from = 0;  // the last binned draw: triangles, first opaque one
  bool opaque_valid = false;
  bool color_valid = false;
  int raster_wpsm = 0;  // RasterParams::warps_per_sm of this context's transparent rasters
  cudaStream_t last_stream = nullptr;
  uint64_t launches = 0;

  // Section timing (oit_profile_*): event pairs recorded around each pass.
  struct Pending {
    int section;
    cudaEvent_t a, b;
  };
  bool prof_on = false;
  std::vector<Pending> prof_pending;
  std::vector<cudaEvent_t> prof_free;
  double prof_ms[OIT_PROF_NUM_SECTIONS] = {};
  uint64_t prof_n[OIT_PROF_NUM_SECTIONS] = {};

  cudaEvent_t prof_event() {
    if (!prof_free.empty()) {
      cudaEvent_t e = prof_free.back();
      prof_free.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  // Returns the start event (or null when profiling is off).
  cudaEvent_t prof_begin(cudaStream_t s) {
    if (!prof_on) return nullptr;
    cudaEvent_t a = prof_event();
    cudaEventRecord(a, s);
    return a;
  }
  void prof_end(int section, cudaEvent_t a, cudaStream_t s) {
    if (!a) return;
    cudaEvent_t b = prof_event();
    cudaEventRecord(b, s);
    prof_pending.push_back({section, a, b});
  }
  int prof_collect() {
    for (const Pending& p : prof_pending) {
      OIT_TRY_CUDA(cudaEventSynchronize(p.b), "profile sync");
      float ms = 0.f;
      OIT_TRY_CUDA(cudaEventElapsedTime(&ms, p.a, p.b), "profile elapsed");
      prof_ms[p.section] += ms;
      prof_n[p.section] += 1;
      prof_free.push_back(p.a);
      prof_free.push_back(p.b);
    }
    prof_pending.clear();
    return OIT_OK;
  }

  ~oit_context() {
    for (const Pending& p : prof_pending) {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    for (cudaEvent_t e : prof_free) cudaEventDestroy(e);
    drop_graph();
    if (graph_stream) cudaStreamDestroy(graph_stream);
    if (graph_in) cudaEventDestroy(graph_in);
    if (graph_out) cudaEventDestroy(graph_out);
    for (PairStat& p : pair_stats) {
      if (p.ev) cudaEventDestroy(p.ev);
      if (p.host_total) cudaFreeHost(p.host_total);
    }
    for (cudaEvent_t e : scene_ev)
      if (e) cudaEventDestroy(e);
    if (scene_ring) cudaFreeHost(scene_ring);
    DevBuf* all[] = {&depth, &opaque_color, &color, &abuf, &aux, &auxdepth, &counter, &accum, &reveal, &out,
                     &out_linear, &err, &frag, &bbox, &setup, &persp, &pair_count, &pair_offset, &scan_tmp, &total,
                     &keys, &tris, &keys_alt, &tris_alt, &hist, &tile_begin, &tile_end, &mesh_v, &mesh_i,
                     &scene_dev, &lens};
    for (DevBuf* b : all) b->release();
  }

  oit::Alg alg() const { return static_cast<oit::Alg>(st.algorithm); }
  bool color_half() const { return (st.flags & OIT_FLAG_HALF_COLOR) != 0; }
  bool arrival() const { return (st.flags & OIT_FLAG_ARRIVAL_ORDER) != 0; }
  size_t color_bytes() const { return color_half() ? 8 : 16; }

  // Views the batched resolve handles: linked list or Loop64, 1x, RGBA8 records.
  bool batch_resolvable() const {
    return (alg() == oit::Alg::LinkedList || alg() == oit::Alg::Loop64) && st.record_format == OIT_RECORD_RGBA8 &&
           S == 1 && ssn == 1 && supersample == 1 && !(st.flags & OIT_FLAG_LINEAR_OUTPUT);
  }
  int lens_stride() const { return (RW + 7) / 8; }
  int lens_rows() const { return (RH + 3) / 4; }
  size_t lens_count() const { return (size_t)lens_stride() * (size_t)lens_rows(); }
  // batched-resolve work items: the 8 micro-tiles of every 16x16 tile
  size_t resolve_items() const { return (size_t)8 * (size_t)num_tiles; }

  // ---- Sample::createFrameImages (oit.cpp:45-220) ----
  int create() {
    OIT_TRY_CUDA(depth.ensure(4), "alloc");
    size_t elems = (size_t)P * ssn;  // A-buffer elements (pixels, or samples with sample shading)
    const bool fp32 = st.record_format == OIT_RECORD_RGBA32F;
    size_t abuf_bytes = 0;
    switch (alg()) {
      case oit::Alg::Simple:
      case oit::Alg::Spinlock:
      case oit::Alg::Interlock:
        abuf_bytes = elems * L * (coverage ? 16 : 8);
        break;
      case oit::Alg::LinkedList:
        abuf_bytes = (size_t)capacity * (fp32 ? 32 : 16);
        break;
      case oit::Alg::Loop:
        abuf_bytes = elems * L * 8;
        break;
      case oit::Alg::Loop64:
        abuf_bytes = elems * L * (fp32 ? 24 : 8);  // keys (+ float4 payloads)
        break;
      default:
        break;
    }
    OIT_TRY_CUDA(abuf.ensure(abuf_bytes), "alloc abuffer");
    OIT_TRY_CUDA(aux.ensure(elems * 4), "alloc aux");
    OIT_TRY_CUDA(auxdepth.ensure(elems * 4), "alloc auxdepth");
    OIT_TRY_CUDA(counter.ensure(4), "alloc counter");
    OIT_TRY_CUDA(color.ensure((size_t)P * ssn * color_bytes()), "alloc color");
    if (alg() == oit::Alg::Weighted) {
      const bool f32 = st.weighted_precision == OIT_WEIGHTED_FP32;
      OIT_TRY_CUDA(accum.ensure((size_t)S * P * (f32 ? 16 : 8)), "alloc accum");
      OIT_TRY_CUDA(reveal.ensure((size_t)S * P * (f32 ? 4 : 2)), "alloc reveal");
    }
    OIT_TRY_CUDA(out.ensure((size_t)W * H * 4), "alloc out");
    OIT_TRY_CUDA(err.ensure(4), "alloc err");
    OIT_TRY_CUDA(frag.ensure(8), "alloc frag");
    OIT_TRY_CUDA(tile_begin.ensure((size_t)2 * num_tiles * 4), "alloc bins");
    OIT_TRY_CUDA(tile_end.ensure((size_t)2 * num_tiles * 4), "alloc bins");
    OIT_TRY_CUDA(total.ensure(4), "alloc total");
    OIT_TRY_CUDA(scene_dev.ensure(kSceneBytes), "alloc scene");
    OIT_TRY_CUDA(cudaMallocHost(&scene_ring, kSceneSlots * kSceneBytes), "alloc pinned scene");
    for (cudaEvent_t& e : scene_ev) OIT_TRY_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
    OIT_TRY_CUDA(cudaMemset(err.p, 0, 4), "memset");
    OIT_TRY_CUDA(cudaMemset(frag.p, 0, 8), "memset");
    OIT_TRY_CUDA(cudaMemset(counter.p, 0, 4), "memset");
    if (batch_resolvable()) {
      OIT_TRY_CUDA(lens.ensure(lens_count()), "alloc lens");
      OIT_TRY_CUDA(cudaMemset(lens.p, 0, lens_count()), "memset");
    }
    return OIT_OK;
  }

  int ensure_opaque_buffers() {
    OIT_TRY_CUDA(depth.ensure((size_t)S * P * 4), "alloc depth");
    OIT_TRY_CUDA(opaque_color.ensure((size_t)S * P * 16), "alloc opaque colour");
    return OIT_OK;
  }

  int ensure_triangles(size_t n) {
    if (n <= tri_cap) return OIT_OK;
    const size_t cap = std::max<size_t>(n, 1024);
    // two records per triangle: the second half of a triangle the near plane
    // splits lives at record count + t
    OIT_TRY_CUDA(bbox.ensure(2 * cap * 8), "alloc bbox");
    OIT_TRY_CUDA(setup.ensure(2 * cap * 96), "alloc setup");
    if (alg() == oit::Alg::Weighted) OIT_TRY_CUDA(persp.ensure(2 * cap * 32), "alloc persp");
    OIT_TRY_CUDA(pair_count.ensure(cap * 4), "alloc pair_count");
    OIT_TRY_CUDA(pair_offset.ensure((cap + 1) * 4), "alloc pair_offset");
    tri_cap = cap;
    return OIT_OK;
  }

  int ensure_pairs(size_t n) {
    if (n > pair_cap || pair_cap == 0) {
      const float scale = st.bin_capacity_scale > 0.0f ? st.bin_capacity_scale : 1.25f;
      const size_t cap = std::max<size_t>((size_t)((double)n * std::max(1.0f, scale)), 4096);
      OIT_TRY_CUDA(keys.ensure(cap * 4), "alloc keys");
      OIT_TRY_CUDA(tris.ensure(cap * 4), "alloc tris");
      OIT_TRY_CUDA(keys_alt.ensure(cap * 4), "alloc keys");
      OIT_TRY_CUDA(tris_alt.ensure(cap * 4), "alloc tris");
      pair_cap = cap;
    }
    const size_t hist_words = oit::radix_hist_words(pair_cap, true);
    OIT_TRY_CUDA(hist.ensure(hist_words * 4), "alloc hist");
    const size_t scan_words = oit::bin_scan_words(tri_cap);
    OIT_TRY_CUDA(scan_tmp.ensure(scan_words * 4), "alloc scan");
    return OIT_OK;
  }

  // oit_update_scene: the newest constants go to the next ring slot, once the
  // copy that last read that slot has run.
  int set_scene(const oit_scene_data* scene) {
    const int k = (scene_slot + 1) % kSceneSlots;
    if (scene_ev_used[k]) OIT_TRY_CUDA(cudaEventSynchronize(scene_ev[k]), "scene slot");
    float* dst = scene_ring + 32 * k;
    std::memcpy(dst, scene->proj_view_matrix, 16 * sizeof(float));
    std::memcpy(dst + 16, scene->view_matrix, 16 * sizeof(float));
    scene_slot = k;
    scene_dirty = true;
    has_scene = true;
    return OIT_OK;
  }

  // Stream-ordered copy of the newest scene constants into scene_dev, before
  // the frame's first kernel; nothing to do when they have not changed. Never
  // captured: a graph reads scene_dev, and this copy precedes its launch.
  int upload_scene(cudaStream_t s) {
    if (!scene_dirty || capturing) return OIT_OK;
    OIT_TRY_CUDA(cudaMemcpyAsync(scene_dev.p, scene_ring + 32 * scene_slot, kSceneBytes, cudaMemcpyHostToDevice, s),
                 "scene h2d");
    OIT_TRY_CUDA(cudaEventRecord(scene_ev[scene_slot], s), "event");
    scene_ev_used[scene_slot] = true;
    scene_dirty = false;
    return OIT_OK;
  }

  oit::SetupParams setup_params(const oit::MeshRef& mesh, uint32_t first, uint32_t count, uint32_t opaque_from) {
    oit::SetupParams sp{};
    sp.vertices = mesh.vertices;
    sp.indices = mesh.indices;
    sp.instances = mesh.instances;
    sp.template_triangles = mesh.template_triangles;
    sp.first_triangle = first;
    sp.num_triangles = count;
    sp.scene = scene_dev.as<float>();
    sp.RW = RW;
    sp.RH = RH;
    sp.alpha_min = st.alpha_min;
    sp.alpha_width = st.alpha_width;
    sp.opaque_from = opaque_from;
    sp.samples = S;
    sp.tiles_x = tiles_x;
    sp.num_tiles = num_tiles;
    sp.bbox = bbox.as<uint2>();
    sp.setup = setup.p;
    sp.persp = (alg() == oit::Alg::Weighted && opaque_from > 0) ? persp.p : nullptr;
    sp.pair_count = pair_count.as<uint32_t>();
    return sp;
  }

  oit::Bins bins() {
    oit::Bins b{};
    b.tile_begin = tile_begin.as<uint32_t>();
    b.tile_end = tile_end.as<uint32_t>();
    b.tris = tris.as<uint32_t>();
    b.keys = keys.as<uint32_t>();
    b.tris_alt = tris_alt.as<uint32_t>();
    b.keys_alt = keys_alt.as<uint32_t>();
    b.pair_offset = pair_offset.as<uint32_t>();
    b.scan_tmp = scan_tmp.as<uint32_t>();
    b.hist = hist.as<uint32_t>();
    b.total = total.as<uint32_t>();
    b.capacity = pair_cap;
    // measured: the 64-view batch 18.64 ms at 8M against 18.96 at 1M; a
    // 2560x1440 MSAA-8 frame alone 6.38 ms at 1M against 6.51 at 8M
    b.sort_direct_max = in_batch ? (8u << 20) : (1u << 20);
    return b;
  }

  // Pair-count history per draw signature: the first draw of a signature reads
  // its pair count back synchronously to size the bins; later draws run without
  // a host round trip, sized from earlier frames (their counts are copied back
  // asynchronously into pinned memory and picked up when ready).
  struct PairStat {
    uint64_t key = 0;
    uint32_t known = 0;
    uint32_t* host_total = nullptr;  // pinned
    cudaEvent_t ev = nullptr;
    bool pending = false;
  };
  std::vector<PairStat> pair_stats;

  PairStat* pair_stat(uint64_t key) {
    for (PairStat& p : pair_stats)
      if (p.key == key) return &p;
    return nullptr;
  }

  // Setup + binning of one draw; afterwards tile_begin/tile_end/tris describe it.
  // Triangles [first, first + opaque_from) are transparent, the rest of the
  // range opaque; one setup, scan and sort bins both kinds.
  int bin(const oit::MeshRef& mesh, uint32_t first, uint32_t count, uint32_t opaque_from, cudaStream_t s) {
    int r = upload_scene(s);
    if (r != OIT_OK) return r;
    r = ensure_triangles(count);
    if (r != OIT_OK) return r;
    if (arrival() && opaque_from == count) {
      // an arrival-order draw without opaque triangles reads only the setup
      // records and bboxes: no tile bins
      oit::SetupParams sp = setup_params(mesh, first, count, opaque_from);
      bin_tris = count;
      bin_opaque_from = opaque_from;
      OIT_TRY_CUDA(oit::bin_setup_only(sp, s, &launches), "setup");
      return OIT_OK;
    }
    const uint64_t key = ((uint64_t)first << 32) ^ ((uint64_t)count << 1) ^ ((uint64_t)opaque_from * 0x9E3779B1ull) ^
                         ((uint64_t)(uintptr_t)mesh.indices << 7) ^ ((uint64_t)(uintptr_t)mesh.instances << 3);
    PairStat* ps = pair_stat(key);
    if (ps && ps->pending && !capturing && cudaEventQuery(ps->ev) == cudaSuccess) {
      ps->known = std::max(ps->known, *ps->host_total);
      ps->pending = false;
    }
    r = ensure_pairs(ps ? ps->known : 0);
    if (r != OIT_OK) return r;
    oit::SetupParams sp = setup_params(mesh, first, count, opaque_from);
    bin_tris = count;
    bin_opaque_from = opaque_from;
    oit::Bins b = bins();
    OIT_TRY_CUDA(oit::bin_setup_scan(sp, b, s, &launches), "bin_setup_scan");
    if (!ps) {
      if (capturing) return OIT_ERR_STATE;  // a captured frame never sizes bins
      // first draw of this signature: size the bins exactly
      PairStat st;
      st.key = key;
      OIT_TRY_CUDA(cudaMallocHost(&st.host_total, 4), "alloc pinned");
      OIT_TRY_CUDA(cudaEventCreateWithFlags(&st.ev, cudaEventDisableTiming), "event");
      OIT_TRY_CUDA(cudaMemcpyAsync(st.host_total, total.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
      OIT_TRY_CUDA(cudaStreamSynchronize(s), "sync");
      st.known = *st.host_total;
      pair_stats.push_back(st);
      ps = &pair_stats.back();
      r = ensure_pairs(ps->known);
      if (r != OIT_OK) return r;
      b = bins();
    }
    OIT_TRY_CUDA(oit::bin_sort(sp, b, key_bits, num_tiles, err.as<uint32_t>(), s, &launches), "bin_sort");
    // bin_sort may have swapped the ping-pong buffers
    if (b.keys != keys.as<uint32_t>()) {
      std::swap(keys, keys_alt);
      std::swap(tris, tris_alt);
    }
    if (!ps->pending || capturing) {
      OIT_TRY_CUDA(cudaMemcpyAsync(ps->host_total, total.p, 4, cudaMemcpyDeviceToHost, s), "d2h");
      if (!capturing) {
        OIT_TRY_CUDA(cudaEventRecord(ps->ev, s), "event");
        ps->pending = true;
      }
    }
    if (capturing) graph_stats.push_back(ps->key);
    return OIT_OK;
  }

  oit::RasterParams raster_params(int tile_offset) {
    oit::RasterParams p{};
    p.RW = RW;
    p.RH = RH;
    p.tiles_x = tiles_x;
    p.tiles_y = tiles_y;
    p.P = P;
    p.S = ssn > 1 ? 1 : S;
    p.ssn = ssn;
    p.L = L;
    p.tail = st.tail_blend ? 1 : 0;
    p.coverage = coverage;
    p.tile_begin = tile_begin.as<uint32_t>();
    p.tile_end = tile_end.as<uint32_t>();
    p.tile_offset = tile_offset;
    p.pair_total = total.as<uint32_t>();
    p.pair_offset = pair_offset.as<uint32_t>();
    p.pair_count = pair_count.as<uint32_t>();
    p.pair_capacity = (uint32_t)std::min<size_t>(pair_cap, 0xFFFFFFFFu);
    p.num_tris = bin_tris;
    p.pass_first = tile_offset != 0 ? 0u : bin_opaque_from;
    p.pass_end = tile_offset != 0 ? bin_opaque_from : bin_tris;
    p.tile_tris = tris.as<uint32_t>();
    p.tile_keys = keys.as<uint32_t>();
    p.bbox = bbox.as<uint2>();
    p.setup = setup.p;
    p.persp = persp.p;
    p.depth = depth.as<uint32_t>();
    p.opaque_color = opaque_color.as<float4>();
    p.has_opaque = opaque_valid ? 1 : 0;
    p.background = background;
    p.color = color.as<float4>();
    p.color_half = color_half() ? 1 : 0;
    p.abuf = abuf.as<uint32_t>();
    p.aux = aux.as<uint32_t>();
    p.auxdepth = auxdepth.as<uint32_t>();
    p.counter = counter.as<uint32_t>();
    p.capacity = capacity;
    p.record_fp32 = st.record_format == OIT_RECORD_RGBA32F;
    p.accum = accum.p;
    p.reveal = reveal.p;
    p.weighted_fp32 = st.weighted_precision == OIT_WEIGHTED_FP32;
    p.error = err.as<uint32_t>();
    p.frag_count = frag.as<unsigned long long>();
    p.warps_per_sm = raster_wpsm;
    if (tile_offset != 0 && batch_resolvable()) {
      p.lens = lens.as<uint8_t>();
      p.lens_stride = lens_stride();
    }
    return p;
  }

  // The batched resolve's descriptor of this context's current frame.
  oit::ResolveView resolve_view(uint8_t* out_dev) const {
    oit::ResolveView v{};
    v.abuf = abuf.as<uint32_t>();
    v.aux = aux.as<uint32_t>();
    v.color = color.as<float4>();
    v.color_half = color_half() ? 1 : 0;
    v.out = out_dev ? out_dev : out.as<uint8_t>();
    v.out_linear = nullptr;
    v.lens = lens.as<uint8_t>();
    v.P = P;
    v.capacity = capacity;
    v.W = RW;
    v.H = RH;
    v.L = L;
    v.kind = alg() == oit::Alg::LinkedList ? oit::kResolveList : oit::kResolveLoop64;
    v.tail = st.tail_blend ? 1 : 0;
    v.mtx = lens_stride();
    v.mty = lens_rows();
    v.tiles_x = tiles_x;
    v.ptx = 2 * tiles_x;
    v.tx_recip = ((1ull << 40) + (uint64_t)v.tiles_x - 1) / (uint64_t)v.tiles_x;  // exact: tiles_x <= 1024
    v.ptx_recip = ((1ull << 40) + (uint64_t)v.ptx - 1) / (uint64_t)v.ptx;
    return v;
  }

  int raster(oit::Alg a, oit::RasterParams& p, cudaStream_t s) {
    cudaError_t e;
    switch (a) {
      case oit::Alg::Simple:
      case oit::Alg::LinkedList:
      case oit::Alg::Opaque: e = oit::launch_raster_a(a, p, s); break;
      case oit::Alg::Loop:
      case oit::Alg::Loop64: e = oit::launch_raster_b(a, p, s); break;
      default: e = oit::launch_raster_c(a, p, s); break;
    }
    ++launches;
    return cuda_status(e, "raster");
  }

  // ---- the transparent pass ----
  int begin_frame(cudaStream_t s) {
    last_stream = s;
    opaque_valid = false;
    color_valid = false;
    return OIT_OK;
  }

  // clearTransparent* (oitRender.cpp:156-356). Only the linked-list counter
  // needs clearing: the COLOR pass writes every pixel's aux words, k-buffer
  // layers and WBOIT accumulators itself.
  int clear_transparent(cudaStream_t s) {
    last_stream = s;
    OIT_TRY_CUDA(cudaMemsetAsync(frag.p, 0, 8, s), "clear");
    if (alg() == oit::Alg::LinkedList) OIT_TRY_CUDA(cudaMemsetAsync(counter.p, 0, 4, s), "clear");
    return OIT_OK;
  }

  int draw_opaque(const oit::MeshRef& mesh, uint32_t first, uint32_t count, cudaStream_t s) {
    last_stream = s;
    int r = clear_opaque_targets(s);
    if (r != OIT_OK) return r;
    if (!count) return OIT_OK;
    cudaEvent_t t0 = prof_begin(s);
    r = bin(mesh, first, count, 0u, s);
    if (r != OIT_OK) return r;
    prof_end(OIT_PROF_OPAQUE_BIN, t0, s);
    return raster_opaque(s);
  }

  int clear_opaque_targets(cudaStream_t s) {
    int r = ensure_opaque_buffers();
    if (r != OIT_OK) return r;
    if (!opaque_valid) {
      OIT_TRY_CUDA(oit::launch_fill_u32(depth.as<uint32_t>(), 0x3F800000u, (size_t)S * P, s), "fill");
      OIT_TRY_CUDA(oit::launch_fill_f4(opaque_color.as<float4>(), background, (size_t)S * P, s), "fill");
      launches += 2;
      opaque_valid = true;
    }
    return OIT_OK;
  }

  oit::RasterParams opaque_pass_params() {
    oit::RasterParams p = raster_params(0);
    p.S = S;    // the opaque pass always tests every sample of a pixel
    p.ssn = 1;
    return p;
  }

  int raster_opaque(cudaStream_t s) {
    oit::RasterParams p = opaque_pass_params();
    cudaEvent_t t1 = prof_begin(s);
    const int r = raster(oit::Alg::Opaque, p, s);
    prof_end(OIT_PROF_OPAQUE_RASTER, t1, s);
    return r;
  }

  // The arrival-order linked-list COLOR pass (OIT_FLAG_ARRIVAL_ORDER).
  int raster_arrival(cudaStream_t s) {
    oit::ArrivalParams a{};
    a.RW = RW;
    a.RH = RH;
    a.P = P;
    a.num_tris = bin_opaque_from;  // the draw's transparent triangles
    a.second_base = bin_tris;
    a.bbox = bbox.as<uint2>();
    a.setup = setup.p;
    a.depth = depth.as<uint32_t>();
    a.opaque_color = opaque_color.as<float4>();
    a.has_opaque = opaque_valid ? 1 : 0;
    a.background = background;
    a.color = color.as<float4>();
    a.color_half = color_half() ? 1 : 0;
    a.pool = abuf.as<uint32_t>();
    a.heads = aux.as<uint32_t>();
    a.counter = counter.as<uint32_t>();
    a.capacity = capacity;
    a.locks = auxdepth.as<uint32_t>();
    a.held_lock = debug_held_lock;
    a.tail = st.tail_blend ? 1 : 0;
    a.error = err.as<uint32_t>();
    a.frag_count = frag.as<unsigned long long>();
    // the batched resolve's per-micro-tile list lengths are not counted: the
    // most any list may hold
    if (batch_resolvable()) OIT_TRY_CUDA(cudaMemsetAsync(lens.p, 0xFF, lens_count(), s), "lens");
    cudaEvent_t t1 = prof_begin(s);
    const cudaError_t e = oit::launch_arrival_ll(a, s, &launches);
    prof_end(OIT_PROF_TRANSPARENT_RASTER, t1, s);
    if (e == cudaSuccess) color_valid = true;
    return cuda_status(e, "arrival raster");
  }

  int raster_transparent(cudaStream_t s) {
    if (arrival()) return raster_arrival(s);
    oit::RasterParams p = raster_params(num_tiles);
    cudaEvent_t t1 = prof_begin(s);
    const int r = raster(alg(), p, s);
    prof_end(OIT_PROF_TRANSPARENT_RASTER, t1, s);
    if (r == OIT_OK) color_valid = true;
    return r;
  }

  int draw_transparent_color(const oit::MeshRef& mesh, uint32_t first, uint32_t count, cudaStream_t s) {
    last_stream = s;
    cudaEvent_t t0 = prof_begin(s);
    int r = bin(mesh, first, count, count, s);
    if (r != OIT_OK) return r;
    prof_end(OIT_PROF_TRANSPARENT_BIN, t0, s);
    return raster_transparent(s);
  }

  oit::CompositeParams composite_params(uint8_t* out_dev) {
    oit::CompositeParams c{};
    c.W = W;
    c.H = H;
    c.RW = RW;
    c.RH = RH;
    c.ss = supersample;
    c.P = P;
    c.S = S;
    c.ssn = ssn;
    c.L = L;
    c.tail = st.tail_blend ? 1 : 0;
    c.coverage = coverage;
    c.record_fp32 = st.record_format == OIT_RECORD_RGBA32F;
    c.weighted_fp32 = st.weighted_precision == OIT_WEIGHTED_FP32;
    c.capacity = capacity;
    c.abuf = abuf.as<uint32_t>();
    c.aux = aux.as<uint32_t>();
    c.color = color.as<float4>();
    c.color_half = color_half() ? 1 : 0;
    c.opaque_color = opaque_color.as<float4>();
    c.has_opaque = opaque_valid ? 1 : 0;
    c.background = background;
    c.accum = accum.p;
    c.reveal = reveal.p;
    c.out_rgba8 = out_dev;
    c.out_linear = nullptr;
    return c;
  }

  int composite(uint8_t* out_dev, cudaStream_t s) {
    last_stream = s;
    if (!color_valid) return OIT_ERR_STATE;
    oit::CompositeParams c = composite_params(out_dev ? out_dev : out.as<uint8_t>());
    if (st.flags & OIT_FLAG_LINEAR_OUTPUT) {
      OIT_TRY_CUDA(out_linear.ensure((size_t)W * H * 16), "alloc linear");
      c.out_linear = out_linear.as<float4>();
    }
    ++launches;
    cudaEvent_t t0 = prof_begin(s);
    const int r = cuda_status(oit::launch_composite(alg(), c, s), "composite");
    prof_end(OIT_PROF_COMPOSITE, t0, s);
    return r;
  }

  // FP64 verification resolve of the current frame (not part of a frame).
  int verify_composite_fp64(double* out_linear_dev, uint8_t* out_rgba8_dev, cudaStream_t s) {
    if (!color_valid) return OIT_ERR_STATE;
    last_stream = s;
    const oit::CompositeParams c = composite_params(out_rgba8_dev);
    ++launches;
    return cuda_status(oit::launch_composite_fp64(alg(), c, out_linear_dev, s), "composite fp64");
  }

  // Sample::onRender, oitRender.cpp:43-153. The transparent objects are the
  // first percent_transparent% of the mesh and the opaque ones the rest, so one
  // binning pass serves both the opaque and the transparent raster.
  // raster = false (a batch whose rasters run as multi-view launches): the
  // frame stops after binning; frame_has_opaque tells whether it has an opaque pass.
  bool frame_has_opaque = false;
  int render_frame_body(const oit::MeshRef& mesh, uint32_t tpo, int32_t percent, uint8_t* out_dev, cudaStream_t s,
                        bool resolve = true, bool raster = true) {
    const uint32_t num_objects = mesh.num_triangles / tpo;
    uint32_t num_transparent = (uint32_t)(((uint64_t)num_objects * (uint32_t)percent) / 100u);
    if (num_transparent > num_objects) num_transparent = num_objects;
    const uint32_t num_opaque = num_objects - num_transparent;
    const uint32_t nt = num_transparent * tpo, total_tris = num_objects * tpo;
    int r = begin_frame(s);
    if (r == OIT_OK) r = clear_transparent(s);
    if (r == OIT_OK && num_opaque > 0) r = clear_opaque_targets(s);
    if (r != OIT_OK) return r;
    cudaEvent_t t0 = prof_begin(s);
    r = bin(mesh, 0, total_tris, nt, s);
    if (r != OIT_OK) return r;
    prof_end(OIT_PROF_TRANSPARENT_BIN, t0, s);
    frame_has_opaque = num_opaque > 0;
    if (!raster) {
      color_valid = true;  // the batch's multi-view rasters follow in the same graph
      return OIT_OK;
    }
    if (num_opaque > 0) r = raster_opaque(s);
    if (r == OIT_OK) r = raster_transparent(s);
    if (r == OIT_OK && resolve) r = composite(out_dev, s);
    return r;
  }

  // ---- CUDA graph of a whole frame (OIT_FLAG_CUDA_GRAPH) ----
  bool capturing = false;
  bool in_batch = false;
  int32_t debug_held_lock = -1;  // oit_debug_hold_arrival_lock  // binning inside a batch graph, beside other views
  cudaGraphExec_t graph_exec = nullptr;
  uint64_t graph_sig = 0;
  uint64_t graph_launches = 0;
  bool graph_opaque_valid = false;
  std::vector<uint64_t> graph_stats;

  // Graphs are captured and replayed on a stream the context owns (the legacy
  // default stream cannot be captured); events order it after and before the
  // caller's stream.
  cudaStream_t graph_stream = nullptr;
  cudaEvent_t graph_in = nullptr, graph_out = nullptr;

  void drop_graph() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
    graph_sig = 0;
  }

  int ensure_graph_stream() {
    if (graph_stream) return OIT_OK;
    OIT_TRY_CUDA(cudaStreamCreateWithFlags(&graph_stream, cudaStreamNonBlocking), "stream");
    OIT_TRY_CUDA(cudaEventCreateWithFlags(&graph_in, cudaEventDisableTiming), "event");
    OIT_TRY_CUDA(cudaEventCreateWithFlags(&graph_out, cudaEventDisableTiming), "event");
    return OIT_OK;
  }

  // Pair counts copied back by a graph replay become known once their event
  // completes; returns false when a bin outgrew its capacity (the graph that
  // reads these bins must be re-captured).
  bool graph_bins_fit() {
    bool fit = true;
    for (uint64_t k : graph_stats) {
      PairStat* ps = pair_stat(k);
      if (ps && ps->pending && cudaEventQuery(ps->ev) == cudaSuccess) {
        ps->known = std::max(ps->known, *ps->host_total);
        ps->pending = false;
      }
      if (ps && ps->known > pair_cap) fit = false;
    }
    return fit;
  }

  int after_graph_launch(cudaStream_t s) {
    for (uint64_t k : graph_stats) {
      PairStat* ps = pair_stat(k);
      if (ps && !ps->pending) {
        OIT_TRY_CUDA(cudaEventRecord(ps->ev, s), "event");
        ps->pending = true;
      }
    }
    return OIT_OK;
  }

  int render_frame(const oit::MeshRef& mesh, uint32_t tpo, int32_t percent, uint8_t* out_dev, cudaStream_t s) {
    if (!tpo || percent < 0) return OIT_ERR_INVALID_ARGUMENT;
    last_stream = s;
    if (!(st.flags & OIT_FLAG_CUDA_GRAPH) || prof_on) return render_frame_body(mesh, tpo, percent, out_dev, s);
    uint64_t sig = 1469598103934665603ull;
    const uint64_t parts[] = {(uint64_t)(uintptr_t)mesh.vertices, (uint64_t)(uintptr_t)mesh.indices,
                              (uint64_t)(uintptr_t)mesh.instances, mesh.num_triangles, tpo, (uint64_t)percent,
                              (uint64_t)(uintptr_t)out_dev, (uint64_t)(uintptr_t)s};
    for (uint64_t v : parts) sig = (sig ^ v) * 1099511628211ull;
    // bins that outgrew their capacity since the capture invalidate the graph
    if (!graph_bins_fit()) drop_graph();
    int gr = ensure_graph_stream();
    if (gr != OIT_OK) return gr;
    if (!graph_exec || graph_sig != sig) {
      drop_graph();
      // one plain frame sizes every buffer, then the same frame is captured
      int r = render_frame_body(mesh, tpo, percent, out_dev, s);
      if (r != OIT_OK) return r;
      OIT_TRY_CUDA(cudaStreamSynchronize(s), "sync");
      graph_stats.clear();
      const uint64_t l0 = launches;
      OIT_TRY_CUDA(cudaStreamBeginCapture(graph_stream, cudaStreamCaptureModeRelaxed), "capture");
      capturing = true;
      r = render_frame_body(mesh, tpo, percent, out_dev, graph_stream);
      capturing = false;
      last_stream = s;
      cudaGraph_t g = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(graph_stream, &g);
      if (r != OIT_OK) {
        if (g) cudaGraphDestroy(g);
        return r;
      }
      OIT_TRY_CUDA(ce, "end capture");
      const cudaError_t ie = cudaGraphInstantiate(&graph_exec, g, 0);
      cudaGraphDestroy(g);
      OIT_TRY_CUDA(ie, "instantiate");
      graph_sig = sig;
      graph_opaque_valid = opaque_valid;
      graph_launches = launches - l0;
      launches = l0;
      return OIT_OK;  // the plain frame above produced this call's image
    }
    int ur = upload_scene(s);  // the replay reads the newest scene constants
    if (ur != OIT_OK) return ur;
    OIT_TRY_CUDA(cudaEventRecord(graph_in, s), "event");
    OIT_TRY_CUDA(cudaStreamWaitEvent(graph_stream, graph_in, 0), "wait");
    OIT_TRY_CUDA(cudaGraphLaunch(graph_exec, graph_stream), "graph launch");
    OIT_TRY_CUDA(cudaEventRecord(graph_out, graph_stream), "event");
    OIT_TRY_CUDA(cudaStreamWaitEvent(s, graph_out, 0), "wait");
    launches += graph_launches;
    int ar = after_graph_launch(graph_stream);
    if (ar != OIT_OK) return ar;
    opaque_valid = graph_opaque_valid;  // as left by the captured frame
    color_valid = true;
    return OIT_OK;
  }
};

// A batch of views rendered as one CUDA graph: the views' frames are captured
// on forked streams so the GPU runs them concurrently (small views alone leave
// most of the 152 SMs idle) and the whole batch costs one graph launch.
struct oit_batch {
  cudaStream_t stream = nullptr;
  std::vector<cudaStream_t> lanes;
  cudaEvent_t fork = nullptr, in = nullptr, out = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t exec = nullptr;
  uint64_t sig = 0;
  uint64_t graph_launches = 0;
  std::vector<oit_context*> ctxs;
  std::vector<bool> opaque_valid;

  // Batched resolve of the views that allow it (oit_context::batch_resolvable),
  // in two parts, linked-list views and Loop64 views, each with its view
  // descriptors, binned work list and the launch shape picked by timing
  // candidates on the batch's own frames; the parts run side by side.
  struct ResolvePart {
    DevBuf views, base, hist, items;
    oit::ResolveBatch rb{};
    int variant = 0, threads = 128, blocks = 0, order = 0, edges = 0;
    bool binned = false;
  };
  ResolvePart rparts[2];
  // shapes pinned by oit_batch_set_resolve_config (blocks 0: all that fit)
  struct Pin {
    bool set = false;
    int variant = 0, threads = 128, blocks = 0, order = 0, edges = 0;
    bool binned = false;
  };
  Pin pin[2];
  // share of its resident blocks the linked-list part launches while the
  // Loop64 part takes the rest (both run side by side); 1 = both full
  float r_share = 1.0f;
  uint64_t rsig = 0;
  bool r_tuned = false;
  // tile rasters: multi-view launches or one per view and pass, and the 1x
  // register budget (warps per SM, 0 = default); pinned, or picked by timing
  // the candidates when a graph is captured
  bool raster_pinned = false;
  oit_raster_config raster_pin{};
  oit_raster_config raster_cfg{};
  bool raster_known = false;
  // each view's frame time on the batch's first (one by one) frames: the
  // longest-first lane order's weights
  std::vector<float> view_ms;
  int num_sms = 0;
  cudaEvent_t rfork = nullptr, rjoin[2] = {nullptr, nullptr};

  void drop() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    sig = 0;
  }
  ~oit_batch() {
    drop();
    for (ResolvePart& rp : rparts) {
      rp.views.release();
      rp.base.release();
      rp.hist.release();
      rp.items.release();
    }
    for (cudaEvent_t e : {rfork, rjoin[0], rjoin[1]})
      if (e) cudaEventDestroy(e);
    for (cudaStream_t l : lanes) cudaStreamDestroy(l);
    for (cudaEvent_t e : joins) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (in) cudaEventDestroy(in);
    if (out) cudaEventDestroy(out);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

bool pow2_layers(uint32_t l) { return l == 1 || l == 2 || l == 4 || l == 8 || l == 16 || l == 32; }

// State::recomputeAntialiasingSettings (oit.h:84-115)
bool aa_settings(uint32_t aa, int* msaa, int* sample_shading, int* supersample) {
  *sample_shading = 0;
  *supersample = 1;
  switch (aa) {
    case OIT_AA_NONE: *msaa = 1; return true;
    case OIT_AA_MSAA_4X: *msaa = 4; return true;
    case OIT_AA_SSAA_4X: *msaa = 4; *sample_shading = 1; return true;
    case OIT_AA_SUPER_4X: *msaa = 1; *supersample = 2; return true;
    case OIT_AA_MSAA_8X: *msaa = 8; return true;
    case OIT_AA_SSAA_8X: *msaa = 8; *sample_shading = 1; return true;
    default: return false;
  }
}

int validate(const oit_state* s, int* msaa, int* ss, int* sup) {
  if (!s) return OIT_ERR_INVALID_ARGUMENT;
  if (s->algorithm >= OIT_NUM_ALGORITHMS) return OIT_ERR_INVALID_ARGUMENT;
  if (!pow2_layers(s->oit_layers)) return OIT_ERR_INVALID_ARGUMENT;
  if (!aa_settings(s->aa_type, msaa, ss, sup)) return OIT_ERR_INVALID_ARGUMENT;
  if (s->width == 0 || s->height == 0) return OIT_ERR_INVALID_ARGUMENT;
  if ((uint64_t)s->width * *sup > 16384 || (uint64_t)s->height * *sup > 16384) return OIT_ERR_INVALID_ARGUMENT;
  if (s->algorithm == OIT_LINKEDLIST && s->linked_list_allocated_per_element < 1) return OIT_ERR_INVALID_ARGUMENT;
  if (s->record_format > OIT_RECORD_RGBA32F || s->weighted_precision > OIT_WEIGHTED_FP32)
    return OIT_ERR_INVALID_ARGUMENT;
  if (!std::isfinite(s->alpha_min) || !std::isfinite(s->alpha_width)) return OIT_ERR_INVALID_ARGUMENT;
  if (s->flags & OIT_FLAG_ARRIVAL_ORDER) {
    // the arrival-order pass: linked list, one sample per pixel, RGBA8 nodes
    if (s->algorithm != OIT_LINKEDLIST || *msaa != 1 || *ss || s->record_format != OIT_RECORD_RGBA8)
      return OIT_ERR_UNSUPPORTED;
  }
  if (s->record_format == OIT_RECORD_RGBA32F) {
    // float records exist for the linked list and Loop64 (whose float payloads
    // take 24 bytes of shared memory per layer and lane: 24 KB per warp at 32
    // layers)
    if (s->algorithm != OIT_LINKEDLIST && s->algorithm != OIT_LOOP64) return OIT_ERR_UNSUPPORTED;
  }
  return OIT_OK;
}

// Descriptors of the batch's resolvable views, rebuilt when the set of views
// (contexts and outputs) changes. Synchronous: never called under capture.
int batch_prepare_resolve(oit_batch* b, const oit_view_frame* views, uint32_t n) {
  uint64_t sig = 1469598103934665603ull;
  uint32_t count = 0;
  for (uint32_t i = 0; i < n; ++i) {
    if (!views[i].ctx->batch_resolvable()) continue;
    ++count;
    for (uint64_t x : {(uint64_t)(uintptr_t)views[i].ctx, (uint64_t)(uintptr_t)views[i].out_rgba8_device})
      sig = (sig ^ x) * 1099511628211ull;
  }
  sig ^= count;
  if (sig == b->rsig) return OIT_OK;
  b->rsig = 0;
  b->r_tuned = false;
  b->r_share = 1.0f;
  if (b->num_sms == 0) OIT_TRY_CUDA(cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, 0), "attr");
  for (int part = 0; part < 2; ++part) {
    const int kind = part == 0 ? oit::kResolveList : oit::kResolveLoop64;
    std::vector<oit::ResolveView> hv;
    std::vector<uint32_t> base;
    uint64_t total = 0;
    for (uint32_t i = 0; i < n; ++i) {
      oit_context* c = views[i].ctx;
      if (!c->batch_resolvable()) continue;
      oit::ResolveView v = c->resolve_view(views[i].out_rgba8_device);
      if (v.kind != kind) continue;
        v.tile_base = (uint32_t)total;
      total += c->resolve_items();
      hv.push_back(v);
      base.push_back(v.tile_base);
    }
    if (hv.size() > (size_t)oit::kResolveMaxViews || total > 0xFFFFFFFFull) return OIT_ERR_INVALID_ARGUMENT;
    oit_batch::ResolvePart& rp = b->rparts[part];
    OIT_TRY_CUDA(rp.views.ensure(hv.size() * sizeof(oit::ResolveView)), "alloc resolve");
    OIT_TRY_CUDA(rp.base.ensure(base.size() * 4), "alloc resolve");
    OIT_TRY_CUDA(rp.hist.ensure(2 * oit::kResolveBuckets * 4), "alloc resolve");
    OIT_TRY_CUDA(rp.items.ensure(total * 4), "alloc resolve");
    if (!hv.empty()) {
      OIT_TRY_CUDA(cudaMemcpy(rp.views.p, hv.data(), hv.size() * sizeof(oit::ResolveView), cudaMemcpyHostToDevice),
                   "h2d");
      OIT_TRY_CUDA(cudaMemcpy(rp.base.p, base.data(), base.size() * 4, cudaMemcpyHostToDevice), "h2d");
    }
    oit::ResolveBatch& rb = rp.rb;
    rb.views = rp.views.as<oit::ResolveView>();
    rb.tile_base = rp.base.as<uint32_t>();
    rb.num_views = (int)hv.size();
    rb.total_tiles = (uint32_t)total;
    rb.hist = rp.hist.as<uint32_t>();
    rb.fill = rb.hist + oit::kResolveBuckets;
    rb.items = rp.items.as<uint32_t>();
    rp.variant = part == 0 ? oit::kResolveVariantList : oit::kResolveVariantLoop64;
  }
  b->rsig = sig;
  return OIT_OK;
}

int part_launch(const oit_batch::ResolvePart& rp, cudaStream_t s, int variant, bool binned, int threads, int blocks,
                int order, int edges, uint64_t* launches) {
  oit::ResolveBatch rb = rp.rb;
  if (rb.num_views == 0) return OIT_OK;
  if (!binned) rb.items = nullptr;
  rb.order = order;
  rb.edges = edges;
  OIT_TRY_CUDA(oit::resolve_bin(rb, s, launches), "resolve bin");
  OIT_TRY_CUDA(oit::resolve_run(rb, variant, threads, blocks, s), "resolve");
  ++*launches;
  return OIT_OK;
}

// Both parts with their tuned shapes, side by side on two of the batch's
// streams, ordered after and before `s`.
int batch_resolve_launch(oit_batch* b, cudaStream_t s, uint64_t* launches) {
  const bool two = b->rparts[0].rb.num_views > 0 && b->rparts[1].rb.num_views > 0 && b->lanes.size() >= 2;
  if (!two) {
    for (const oit_batch::ResolvePart& rp : b->rparts) {
      const int r = part_launch(rp, s, rp.variant, rp.binned, rp.threads, rp.blocks, rp.order, rp.edges, launches);
      if (r != OIT_OK) return r;
    }
    return OIT_OK;
  }
  OIT_TRY_CUDA(cudaEventRecord(b->rfork, s), "event");
  for (int k = 0; k < 2; ++k) {
    const oit_batch::ResolvePart& rp = b->rparts[k];
    OIT_TRY_CUDA(cudaStreamWaitEvent(b->lanes[k], b->rfork, 0), "wait");
    const float share = b->r_share >= 1.0f ? 1.0f : (k == 0 ? b->r_share : 1.0f - b->r_share);
    const int blocks = std::max(1, (int)((float)rp.blocks * share));
    const int r =
        part_launch(rp, b->lanes[k], rp.variant, rp.binned, rp.threads, blocks, rp.order, rp.edges, launches);
    if (r != OIT_OK) return r;
    OIT_TRY_CUDA(cudaEventRecord(b->rjoin[k], b->lanes[k]), "event");
    OIT_TRY_CUDA(cudaStreamWaitEvent(s, b->rjoin[k], 0), "wait");
  }
  return OIT_OK;
}

// The autotuner, per part: kernel variant (linked lists: sort arrays in local
// memory, or the first 8 entries in shared memory; short lists in 4 or 8
// registers; one or two micro-tiles per warp step), block size and binned
// versus view-order
// work lists, each timed with CUDA events on the batch's current frames (the
// resolve only writes the outputs, so reruns are harmless); the grid holds
// every block that fits. The fastest shape is kept for the batch's views.
// Then, with both parts present, the share of the machine each takes when they
// run side by side is timed the same way.
int batch_autotune(oit_batch* b, cudaStream_t s) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  OIT_TRY_CUDA(cudaEventCreate(&e0), "event");
  OIT_TRY_CUDA(cudaEventCreate(&e1), "event");
  int r = OIT_OK;
  uint64_t scratch = 0;
  for (int part = 0; part < 2 && r == OIT_OK; ++part) {
    oit_batch::ResolvePart& rp = b->rparts[part];
    if (rp.rb.num_views == 0) continue;
    if (b->pin[part].set) {
      const oit_batch::Pin& pn = b->pin[part];
      const int bps = oit::resolve_blocks_per_sm(rp.rb, pn.variant, pn.threads);
      if (bps <= 0) {
        r = OIT_ERR_UNSUPPORTED;
        break;
      }
      rp.variant = pn.variant;
      rp.threads = pn.threads;
      rp.blocks = pn.blocks > 0 ? pn.blocks : bps * b->num_sms;
      rp.binned = pn.binned;
      rp.order = pn.order;
      rp.edges = pn.edges;
      continue;
    }
    float best = 1e30f;
    std::vector<int> variants;
    if (part == 0)
      variants = {oit::kResolveVariantList, oit::kResolveVariantListShared, oit::kResolveVariantListx2,
                  oit::kResolveVariantListShort4, oit::kResolveVariantListShort8, oit::kResolveVariantListDense,
                  oit::kResolveVariantListShort8Dense};
    else variants = {oit::kResolveVariantLoop64, oit::kResolveVariantLoop64x2, oit::kResolveVariantLoop64Dense};
    for (int variant : variants) {
      for (int threads : {64, 128, 256}) {
        const int bps = oit::resolve_blocks_per_sm(rp.rb, variant, threads);
        if (bps <= 0) continue;
        const int blocks = bps * b->num_sms;
        for (int order : {0, 1})
          for (int bin_mode : {1, 2, 0}) {  // binned by log2 cost, binned by cost, view order
            const bool binned = bin_mode > 0;
            const int edges = bin_mode == 2 ? 1 : 0;
            r = part_launch(rp, s, variant, binned, threads, blocks, order, edges, &scratch);  // warm-up
            if (r != OIT_OK) break;
            cudaEventRecord(e0, s);
            for (int k = 0; k < 3 && r == OIT_OK; ++k)
              r = part_launch(rp, s, variant, binned, threads, blocks, order, edges, &scratch);
            cudaEventRecord(e1, s);
            if (r != OIT_OK) break;
            if (cudaEventSynchronize(e1) != cudaSuccess) {
              r = OIT_ERR_CUDA;
              break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
              best = ms;
              rp.variant = variant;
              rp.threads = threads;
              rp.blocks = blocks;
              rp.binned = binned;
              rp.order = order;
              rp.edges = edges;
            }
          }
        if (r != OIT_OK) break;
      }
      if (r != OIT_OK) break;
    }
    if (r == OIT_OK && best >= 1e30f) r = OIT_ERR_UNSUPPORTED;
  }
  // both parts together: the share of the machine the linked-list part takes
  if (r == OIT_OK && b->rparts[0].rb.num_views > 0 && b->rparts[1].rb.num_views > 0 && b->lanes.size() >= 2) {
    float best = 1e30f;
    float pick = 1.0f;
    for (float share : {1.0f, 0.7f, 0.5f, 0.3f}) {
      b->r_share = share;
      r = batch_resolve_launch(b, s, &scratch);  // warm-up
      if (r != OIT_OK) break;
      cudaEventRecord(e0, s);
      for (int k = 0; k < 3 && r == OIT_OK; ++k) r = batch_resolve_launch(b, s, &scratch);
      cudaEventRecord(e1, s);
      if (r != OIT_OK) break;
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        r = OIT_ERR_CUDA;
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        pick = share;
      }
    }
    b->r_share = pick;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (r != OIT_OK) return r;
  b->r_tuned = true;
  // leave the outputs written by the chosen shapes
  return batch_resolve_launch(b, s, &scratch);
}

// The tile rasters of a batch as multi-view launches, after every view's
// binning: one launch per (pass, algorithm, sample layout) group and at most
// kMvMaxViews views, the largest views' CTAs first; opaque passes before the
// transparent ones that read their depth.
int batch_mv_rasters(const oit_view_frame* views, uint32_t n, cudaStream_t s, uint64_t* launches) {
  struct Item {
    bool opaque;
    int alg, S, ssn;
    uint64_t size;
    oit_context* c;
  };
  std::vector<Item> items;
  for (uint32_t i = 0; i < n; ++i) {
    oit_context* c = views[i].ctx;
    if (c->frame_has_opaque) items.push_back({true, (int)oit::Alg::Opaque, c->S, 1, (uint64_t)c->P * c->S, c});
    if (!c->arrival()) items.push_back({false, (int)c->alg(), c->ssn > 1 ? 1 : c->S, c->ssn, (uint64_t)c->P * c->ssn, c});
  }
  std::stable_sort(items.begin(), items.end(), [](const Item& a, const Item& b) {
    if (a.opaque != b.opaque) return a.opaque;
    if (a.alg != b.alg) return a.alg < b.alg;
    if (a.S != b.S) return a.S < b.S;
    if (a.ssn != b.ssn) return a.ssn < b.ssn;
    return a.size > b.size;
  });
  std::unique_ptr<oit::MvRaster> mv(new (std::nothrow) oit::MvRaster());
  if (!mv) return OIT_ERR_OUT_OF_MEMORY;
  size_t k = 0;
  while (k < items.size()) {
    const Item& g = items[k];
    mv->n = 0;
    uint32_t ctas = 0;
    while (k < items.size() && mv->n < oit::kMvMaxViews && items[k].opaque == g.opaque && items[k].alg == g.alg &&
           items[k].S == g.S && items[k].ssn == g.ssn) {
      oit_context* c = items[k].c;
      mv->v[mv->n] = g.opaque ? c->opaque_pass_params() : c->raster_params(c->num_tiles);
      ctas += (uint32_t)(c->tiles_x * c->tiles_y * (g.opaque ? 1 : c->ssn) *
                         (oit::kWarpsPerTile / oit::kRasterWarpsPerBlock));
      mv->cta_end[mv->n++] = ctas;
      ++k;
    }
    cudaError_t e;
    const oit::Alg a = static_cast<oit::Alg>(g.alg);
    switch (a) {
      case oit::Alg::Simple:
      case oit::Alg::LinkedList:
      case oit::Alg::Opaque: e = oit::launch_raster_mv_a(a, *mv, s); break;
      case oit::Alg::Loop:
      case oit::Alg::Loop64: e = oit::launch_raster_mv_b(a, *mv, s); break;
      default: e = oit::launch_raster_mv_c(a, *mv, s); break;
    }
    ++*launches;
    if (e != cudaSuccess) return cuda_status(e, "multi-view raster");
  }
  for (uint32_t i = 0; i < n; ++i) {  // arrival-order passes are launched per view
    oit_context* c = views[i].ctx;
    if (!c->arrival()) continue;
    const uint64_t l0 = c->launches;
    const int r = c->raster_arrival(s);
    *launches += c->launches - l0;
    c->launches = l0;
    if (r != OIT_OK) return r;
  }
  return OIT_OK;
}

// Captures the batch's graph: every view's frame on the forked streams (with
// multi_view, only up to its binning; the rasters then run as multi-view
// launches), then the batched resolve. The caller has rendered plain frames
// (buffers sized) and tuned the resolve.
// The capture order of the views and the lane (forked stream) of each:
// round-robin in view order, or longest first (decreasing measured frame
// time, each view to the lane with the least work so far).
void batch_lanes(const oit_batch* b, uint32_t n, int lane_order, std::vector<uint32_t>& order,
                 std::vector<size_t>& lane) {
  const size_t K = b->lanes.size();
  order.resize(n);
  lane.resize(n);
  for (uint32_t i = 0; i < n; ++i) {
    order[i] = i;
    lane[i] = i % K;
  }
  if (lane_order != 1 || b->view_ms.size() != n) return;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return b->view_ms[x] > b->view_ms[y]; });
  std::vector<double> load(K, 0.0);
  for (uint32_t i : order) {
    const size_t k = (size_t)(std::min_element(load.begin(), load.end()) - load.begin());
    lane[i] = k;
    load[k] += b->view_ms[i];
  }
}

int batch_capture(oit_batch* b, const oit_view_frame* views, uint32_t n, cudaStream_t s, bool multi_view,
                  int lane_order, cudaGraphExec_t* exec, uint64_t* launches) {
  *exec = nullptr;
  OIT_TRY_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed), "capture");
  int r = OIT_OK;
  cudaError_t e = cudaEventRecord(b->fork, b->stream);
  const size_t K = b->lanes.size();
  for (size_t k = 0; k < K && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(b->lanes[k], b->fork, 0);
  uint64_t nodes = 0;
  b->ctxs.assign(n, nullptr);
  b->opaque_valid.assign(n, false);
  std::vector<uint32_t> order;
  std::vector<size_t> lane;
  batch_lanes(b, n, lane_order, order, lane);
  for (uint32_t j = 0; j < n && e == cudaSuccess && r == OIT_OK; ++j) {
    const uint32_t i = order[j];
    const oit_view_frame& v = views[i];
    oit_context* c = v.ctx;
    const uint64_t l0 = c->launches;
    c->graph_stats.clear();
    c->capturing = true;
    c->in_batch = true;
    r = c->render_frame_body(view_mesh(v), view_tpo(v), v.percent_transparent, v.out_rgba8_device,
                             b->lanes[lane[i]], !multi_view && !c->batch_resolvable(), !multi_view);
    c->capturing = false;
    c->in_batch = false;
    nodes += c->launches - l0;
    c->launches = l0;
    c->last_stream = s;
    b->ctxs[i] = c;
    b->opaque_valid[i] = c->opaque_valid;
  }
  for (size_t k = 0; k < K && e == cudaSuccess; ++k) {
    e = cudaEventRecord(b->joins[k], b->lanes[k]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->joins[k], 0);
  }
  if (e == cudaSuccess && r == OIT_OK && multi_view) {
    r = batch_mv_rasters(views, n, b->stream, &nodes);
    for (uint32_t i = 0; i < n && r == OIT_OK; ++i) {
      oit_context* c = views[i].ctx;
      if (c->batch_resolvable()) continue;
      const uint64_t l0 = c->launches;
      r = c->composite(views[i].out_rgba8_device, b->stream);
      nodes += c->launches - l0;
      c->launches = l0;
      c->last_stream = s;
    }
  }
  if (e == cudaSuccess && r == OIT_OK) r = batch_resolve_launch(b, b->stream, &nodes);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
  if (r != OIT_OK || e != cudaSuccess || ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (r != OIT_OK) return r;
    return cuda_status(e != cudaSuccess ? e : ce, "batch capture");
  }
  const cudaError_t ie = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  OIT_TRY_CUDA(ie, "batch instantiate");
  *launches = nodes;
  return OIT_OK;
}

// Mean time of `reps` replays of a batch graph (after one warm-up).
int time_graph(cudaGraphExec_t exec, cudaStream_t s, int reps, float* ms) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  OIT_TRY_CUDA(cudaEventCreate(&e0), "event");
  cudaError_t e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
  if (e == cudaSuccess) e = cudaEventRecord(e0, s);
  for (int k = 0; k < reps && e == cudaSuccess; ++k) e = cudaGraphLaunch(exec, s);
  if (e == cudaSuccess) e = cudaEventRecord(e1, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  *ms /= (float)reps;
  return cuda_status(e, "time graph");
}

}  // namespace

extern "C" {

int oit_abuffer_bytes(const oit_state* s, uint64_t* abuffer_bytes, uint64_t* aux_bytes) {
  int msaa, ss, sup;
  if (!s) return OIT_ERR_INVALID_ARGUMENT;
  if (s->algorithm >= OIT_NUM_ALGORITHMS || !pow2_layers(s->oit_layers) || !aa_settings(s->aa_type, &msaa, &ss, &sup))
    return OIT_ERR_INVALID_ARGUMENT;
  // oit.cpp:100-163 and 165-201
  const uint64_t bw = (uint64_t)s->width * sup, bh = (uint64_t)s->height * sup;
  const bool coverage = msaa > 1 && !ss;
  uint64_t per_sample = 0, stride = 0, aux = 0;
  switch (s->algorithm) {
    case OIT_SIMPLE: per_sample = s->oit_layers; stride = coverage ? 16 : 8; aux = 1; break;
    case OIT_SPINLOCK: per_sample = s->oit_layers; stride = coverage ? 16 : 8; aux = 3; break;
    case OIT_INTERLOCK: per_sample = s->oit_layers; stride = coverage ? 16 : 8; aux = 2; break;
    case OIT_LINKEDLIST: per_sample = (uint64_t)std::max(0, s->linked_list_allocated_per_element); stride = 16; aux = 1; break;
    case OIT_LOOP: per_sample = 2ull * s->oit_layers; stride = 4; aux = 1; break;
    case OIT_LOOP64: per_sample = s->oit_layers; stride = 8; aux = 1; break;
    default: break;
  }
  if (ss) per_sample *= (uint64_t)msaa;
  const uint64_t layers = ss ? (uint64_t)msaa : 1;
  if (abuffer_bytes) *abuffer_bytes = bw * bh * per_sample * stride;
  if (aux_bytes) *aux_bytes = bw * bh * 4 * aux * layers + (s->algorithm == OIT_LINKEDLIST ? 4 : 0);
  return OIT_OK;
}

int oit_create(const oit_state* state, oit_context** out_ctx) {
  if (!out_ctx) return OIT_ERR_INVALID_ARGUMENT;
  *out_ctx = nullptr;
  int msaa = 1, ss = 0, sup = 1;
  int r = validate(state, &msaa, &ss, &sup);
  if (r != OIT_OK) return r;
  oit_context* c = new (std::nothrow) oit_context();
  if (!c) return OIT_ERR_OUT_OF_MEMORY;
  c->st = *state;
  c->msaa = msaa;
  c->sample_shading = ss;
  c->supersample = sup;
  c->W = (int)state->width;
  c->H = (int)state->height;
  c->RW = c->W * sup;
  c->RH = c->H * sup;
  c->P = (uint32_t)c->RW * (uint32_t)c->RH;
  c->S = msaa;
  c->coverage = (msaa > 1 && !ss) ? 1 : 0;
  c->ssn = (ss && state->algorithm != OIT_WEIGHTED) ? msaa : 1;
  c->L = (int)state->oit_layers;
  c->tiles_x = (c->RW + oit::kTile - 1) / oit::kTile;
  c->tiles_y = (c->RH + oit::kTile - 1) / oit::kTile;
  c->num_tiles = c->tiles_x * c->tiles_y;
  c->key_bits = 1;
  while ((1 << c->key_bits) < 2 * c->num_tiles) ++c->key_bits;  // opaque and transparent lists
  if (state->algorithm == OIT_LINKEDLIST) {
    // oit.cpp:125 and 148-152: nodes per pixel, per sample with sample shading
    const uint64_t cap = (uint64_t)state->linked_list_allocated_per_element * c->P * c->ssn;
    if (cap >= 0xFFFFFFFFull) {
      delete c;
      return OIT_ERR_INVALID_ARGUMENT;
    }
    c->capacity = (uint32_t)cap;
  }
  r = c->create();
  if (r != OIT_OK) {
    delete c;
    return r;
  }
  *out_ctx = c;
  return OIT_OK;
}

int oit_destroy(oit_context* ctx) {
  if (!ctx) return OIT_ERR_INVALID_ARGUMENT;
  cudaDeviceSynchronize();
  delete ctx;
  return OIT_OK;
}

int oit_update_scene(oit_context* ctx, const oit_scene_data* scene) {
  if (!ctx || !scene) return OIT_ERR_INVALID_ARGUMENT;
  return ctx->set_scene(scene);
}

int oit_begin_frame(oit_context* ctx, void* stream) {
  if (!ctx) return OIT_ERR_INVALID_ARGUMENT;
  return ctx->begin_frame(static_cast<cudaStream_t>(stream));
}

int oit_clear_transparent(oit_context* ctx, void* stream) {
  if (!ctx) return OIT_ERR_INVALID_ARGUMENT;
  return ctx->clear_transparent(static_cast<cudaStream_t>(stream));
}

static bool mesh_ok(const oit_mesh* m, uint32_t first, uint32_t count) {
  if (!m) return false;
  if (count == 0) return true;
  if (!m->vertices_device || !m->indices_device) return false;
  return (uint64_t)first + count <= m->num_triangles;
}

static oit::MeshRef mesh_ref(const oit_mesh* m) {
  return oit::MeshRef{m->vertices_device, m->indices_device, nullptr, m->num_triangles, 0};
}

// Template and instance table present, instance table 16-byte aligned (it is
// read as float4), frame triangle count within 32 bits.
static bool instanced_ok(const oit_instanced_mesh* m) {
  if (!m || !m->template_vertices_device || !m->template_indices_device || !m->instances_device) return false;
  if (!m->template_vertices || !m->template_triangles || !m->num_instances) return false;
  if ((uintptr_t)m->instances_device % 16 != 0) return false;
  return (uint64_t)m->template_triangles * m->num_instances <= 0xFFFFFFFFull / 3;
}

static oit::MeshRef instanced_ref(const oit_instanced_mesh* m) {
  return oit::MeshRef{m->template_vertices_device, m->template_indices_device, m->instances_device,
                      m->template_triangles * m->num_instances, m->template_triangles};
}

int oit_draw_opaque(oit_context* ctx, const oit_mesh* mesh, uint32_t first, uint32_t count, void* stream) {
  if (!ctx || !mesh_ok(mesh, first, count)) return OIT_ERR_INVALID_ARGUMENT;
  if (!ctx->has_scene) return OIT_ERR_STATE;
  return ctx->draw_opaque(mesh_ref(mesh), first, count, static_cast<cudaStream_t>(stream));
}

int oit_draw_transparent_color(oit_context* ctx, const oit_mesh* mesh, uint32_t first, uint32_t count, void* stream) {
  if (!ctx || !mesh_ok(mesh, first, count)) return OIT_ERR_INVALID_ARGUMENT;
  if (!ctx->has_scene) return OIT_ERR_STATE;
  return ctx->draw_transparent_color(mesh_ref(mesh), first, count, static_cast<cudaStream_t>(stream));
}

int oit_composite(oit_context* ctx, uint8_t* out, void* stream) {
  if (!ctx) return OIT_ERR_INVALID_ARGUMENT;
  return ctx->composite(out, static_cast<cudaStream_t>(stream));
}

int oit_verify_composite_fp64(oit_context* ctx, double* out_linear, uint8_t* out_rgba8, void* stream) {
  if (!ctx || (!out_linear && !out_rgba8)) return OIT_ERR_INVALID_ARGUMENT;
  return ctx->verify_composite_fp64(out_linear, out_rgba8, static_cast<cudaStream_t>(stream));
}

int oit_draw_transparent(oit_context* ctx, const oit_mesh* mesh, uint32_t num_triangles, uint8_t* out, void* stream) {
  int r = oit_draw_transparent_color(ctx, mesh, 0, num_triangles, stream);
  if (r != OIT_OK) return r;
  return oit_composite(ctx, out, stream);
}

int oit_render_frame(oit_context* ctx, const oit_mesh* mesh, uint32_t tpo, int32_t percent, uint8_t* out,
                     void* stream) {
  if (!ctx || !mesh) return OIT_ERR_INVALID_ARGUMENT;
  if (!ctx->has_scene) return OIT_ERR_STATE;
  if (!mesh_ok(mesh, 0, mesh->num_triangles)) return OIT_ERR_INVALID_ARGUMENT;
  return ctx->render_frame(mesh_ref(mesh), tpo, percent, out, static_cast<cudaStream_t>(stream));
}

int oit_render_frame_host(oit_context* ctx, const float* vertices, uint32_t num_vertices, const uint32_t* indices,
                          uint32_t num_triangles, uint32_t tpo, int32_t percent, uint8_t* out_host, void* stream) {
  if (!ctx || !vertices || !indices || !out_host || !num_vertices) return OIT_ERR_INVALID_ARGUMENT;
  if (!ctx->has_scene) return OIT_ERR_STATE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t vb = (size_t)num_vertices * 40, ib = (size_t)num_triangles * 12;
  OIT_TRY_CUDA(ctx->mesh_v.ensure(vb), "alloc mesh");
  OIT_TRY_CUDA(ctx->mesh_i.ensure(ib), "alloc mesh");
  OIT_TRY_CUDA(cudaMemcpyAsync(ctx->mesh_v.p, vertices, vb, cudaMemcpyHostToDevice, s), "h2d");
  OIT_TRY_CUDA(cudaMemcpyAsync(ctx->mesh_i.p, indices, ib, cudaMemcpyHostToDevice, s), "h2d");
  oit_mesh m{ctx->mesh_v.as<float>(), ctx->mesh_i.as<uint32_t>(), num_vertices, num_triangles};
  int r = ctx->render_frame(mesh_ref(&m), tpo, percent, nullptr, s);
  if (r != OIT_OK) return r;
  OIT_TRY_CUDA(cudaMemcpyAsync(out_host, ctx->out.p, (size_t)ctx->W * ctx->H * 4, cudaMemcpyDeviceToHost, s), "d2h");
  OIT_TRY_CUDA(cudaStreamSynchronize(s), "sync");
  return OIT_OK;
}

static oit::MeshRef view_mesh(const oit_view_frame& v) {
  return v.instanced_mesh ? instanced_ref(v.instanced_mesh) : mesh_ref(v.mesh);
}

static uint32_t view_tpo(const oit_view_frame& v) {
  return v.instanced_mesh ? v.instanced_mesh->template_triangles : v.triangles_per_object;
}

int oit_render_frame_instanced(oit_context* ctx, const oit_instanced_mesh* mesh, int32_t percent, uint8_t* out,
                               void* stream) {
  if (!ctx || !instanced_ok(mesh)) return OIT_ERR_INVALID_ARGUMENT;
  if (!ctx->has_scene) return OIT_ERR_STATE;
  return ctx->render_frame(instanced_ref(mesh), mesh->template_triangles, percent, out, static_cast<cudaStream_t>(stream));
}

int oit_render_frame_instanced_host(oit_context* ctx, const float* template_vertices, uint32_t num_template_vertices,
                                    const uint32_t* template_indices, uint32_t num_template_triangles,
                                    const float* instances, uint32_t num_instances, int32_t percent,
                                    uint8_t* out_host, void* stream) {
  if (!ctx || !template_vertices || !template_indices || !instances || !out_host) return OIT_ERR_INVALID_ARGUMENT;
  if (!ctx->has_scene) return OIT_ERR_STATE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // one device buffer: template vertices, instances (16-byte aligned), indices
  const size_t vb = (size_t)num_template_vertices * 24, nb = (size_t)num_instances * 32;
  const size_t ib = (size_t)num_template_triangles * 12;
  const size_t v_pad = (vb + 255) & ~(size_t)255;
  OIT_TRY_CUDA(ctx->mesh_v.ensure(v_pad + nb), "alloc mesh");
  OIT_TRY_CUDA(ctx->mesh_i.ensure(ib), "alloc mesh");
  oit_instanced_mesh m{ctx->mesh_v.as<float>(), ctx->mesh_i.as<uint32_t>(),
                       reinterpret_cast<const float*>(static_cast<char*>(ctx->mesh_v.p) + v_pad),
                       num_template_vertices, num_template_triangles, num_instances};
  if (!instanced_ok(&m)) return OIT_ERR_INVALID_ARGUMENT;
  OIT_TRY_CUDA(cudaMemcpyAsync(ctx->mesh_v.p, template_vertices, vb, cudaMemcpyHostToDevice, s), "h2d");
  OIT_TRY_CUDA(cudaMemcpyAsync(static_cast<char*>(ctx->mesh_v.p) + v_pad, instances, nb, cudaMemcpyHostToDevice, s),
               "h2d");
  OIT_TRY_CUDA(cudaMemcpyAsync(ctx->mesh_i.p, template_indices, ib, cudaMemcpyHostToDevice, s), "h2d");
  int r = ctx->render_frame(instanced_ref(&m), num_template_triangles, percent, nullptr, s);
  if (r != OIT_OK) return r;
  OIT_TRY_CUDA(cudaMemcpyAsync(out_host, ctx->out.p, (size_t)ctx->W * ctx->H * 4, cudaMemcpyDeviceToHost, s), "d2h");
  OIT_TRY_CUDA(cudaStreamSynchronize(s), "sync");
  return OIT_OK;
}

int oit_batch_create(uint32_t parallel_streams, oit_batch** out) {
  if (!out) return OIT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const uint32_t n = parallel_streams ? std::min<uint32_t>(parallel_streams, 64) : 8;
  oit_batch* b = new (std::nothrow) oit_batch();
  if (!b) return OIT_ERR_OUT_OF_MEMORY;
  auto fail = [&](cudaError_t e) {
    delete b;
    return cuda_status(e, "batch create");
  };
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(e);
  for (uint32_t i = 0; i < n; ++i) {
    cudaStream_t l = nullptr;
    cudaEvent_t j = nullptr;
    if ((e = cudaStreamCreateWithFlags(&l, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
    b->lanes.push_back(l);
    if ((e = cudaEventCreateWithFlags(&j, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
    b->joins.push_back(j);
  }
  for (cudaEvent_t* ev : {&b->fork, &b->in, &b->out, &b->rfork, &b->rjoin[0], &b->rjoin[1]})
    if ((e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming)) != cudaSuccess) return fail(e);
  *out = b;
  return OIT_OK;
}

int oit_batch_destroy(oit_batch* b) {
  if (!b) return OIT_ERR_INVALID_ARGUMENT;
  cudaDeviceSynchronize();
  delete b;
  return OIT_OK;
}

int oit_batch_launch_count(oit_batch* b, uint64_t* launches) {
  if (!b || !launches) return OIT_ERR_INVALID_ARGUMENT;
  *launches = b->graph_launches;
  return OIT_OK;
}

int oit_batch_render(oit_batch* b, const oit_view_frame* views, uint32_t n, void* stream) {
  if (!b || !views || n == 0) return OIT_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  uint64_t sig = 1469598103934665603ull;
  for (uint32_t i = 0; i < n; ++i) {
    const oit_view_frame& v = views[i];
    if (!v.ctx || v.percent_transparent < 0) return OIT_ERR_INVALID_ARGUMENT;
    if (v.instanced_mesh ? !instanced_ok(v.instanced_mesh) : (!v.mesh || !v.triangles_per_object))
      return OIT_ERR_INVALID_ARGUMENT;
    if (!v.ctx->has_scene) return OIT_ERR_STATE;
    if (!v.instanced_mesh && !mesh_ok(v.mesh, 0, v.mesh->num_triangles)) return OIT_ERR_INVALID_ARGUMENT;
    for (uint32_t j = 0; j < i; ++j)
      if (views[j].ctx == v.ctx) return OIT_ERR_INVALID_ARGUMENT;  // one frame per context
    const oit::MeshRef m = view_mesh(v);
    const uint64_t parts[] = {(uint64_t)(uintptr_t)v.ctx, (uint64_t)(uintptr_t)m.vertices,
                              (uint64_t)(uintptr_t)m.indices, (uint64_t)(uintptr_t)m.instances, m.num_triangles,
                              view_tpo(v), (uint64_t)v.percent_transparent,
                              (uint64_t)(uintptr_t)v.out_rgba8_device};
    for (uint64_t x : parts) sig = (sig ^ x) * 1099511628211ull;
  }
  sig ^= n;
  bool fit = true;
  for (uint32_t i = 0; i < n; ++i) fit = views[i].ctx->graph_bins_fit() && fit;
  if (!fit || sig != b->sig) b->drop();
  if (!b->exec) {
    // plain frames, one view after the other, size every buffer (and time
    // each view for the longest-first lane order); views the batched resolve
    // handles are resolved together afterwards
    std::vector<cudaEvent_t> marks(n + 1, nullptr);
    auto free_marks = [&]() {
      for (cudaEvent_t ev : marks)
        if (ev) cudaEventDestroy(ev);
    };
    for (cudaEvent_t& ev : marks) {
      const cudaError_t ce = cudaEventCreate(&ev);
      if (ce != cudaSuccess) {
        ev = nullptr;
        free_marks();
        return cuda_status(ce, "event");
      }
    }
    for (uint32_t i = 0; i < n; ++i) {
      const oit_view_frame& v = views[i];
      cudaError_t ce = cudaEventRecord(marks[i], s);
      int r = ce == cudaSuccess ? v.ctx->render_frame_body(view_mesh(v), view_tpo(v), v.percent_transparent,
                                                            v.out_rgba8_device, s, !v.ctx->batch_resolvable())
                                : cuda_status(ce, "event");
      if (r != OIT_OK) {
        free_marks();
        return r;
      }
    }
    {
      const cudaError_t ce = cudaEventRecord(marks[n], s);
      if (ce != cudaSuccess) {
        free_marks();
        return cuda_status(ce, "event");
      }
    }
    int pr = batch_prepare_resolve(b, views, n);
    if (pr != OIT_OK) return pr;
    uint64_t scratch = 0;
    pr = b->r_tuned ? batch_resolve_launch(b, s, &scratch) : batch_autotune(b, s);
    if (pr != OIT_OK) return pr;
    {
      const cudaError_t ce = cudaStreamSynchronize(s);
      if (ce == cudaSuccess) {
        b->view_ms.assign(n, 0.0f);
        for (uint32_t i = 0; i < n; ++i)
          if (cudaEventElapsedTime(&b->view_ms[i], marks[i], marks[i + 1]) != cudaSuccess) b->view_ms[i] = 0.0f;
      }
      free_marks();
      OIT_TRY_CUDA(ce, "sync");
    }
    // the graph: as pinned, or each raster configuration (per-view launches at
    // the default and at the 32-warp register budget, each in both lane
    // orders, multi-view launches) captured and timed on these frames, the
    // fastest kept
    std::vector<oit_raster_config> cands;
    if (b->raster_pinned) cands.push_back(b->raster_pin);
    else
      cands = {oit_raster_config{0, 0, 0}, oit_raster_config{0, 0, 1}, oit_raster_config{0, 32, 0},
               oit_raster_config{0, 32, 1}, oit_raster_config{1, 0, 0}};
    cudaGraphExec_t best = nullptr;
    uint64_t best_launches = 0;
    float best_ms = 1e30f;
    oit_raster_config best_cfg{};
    for (const oit_raster_config& cfg : cands) {
      cudaGraphExec_t ex = nullptr;
      uint64_t nodes = 0;
      std::vector<int> saved(n);
      for (uint32_t i = 0; i < n; ++i) {  // the budget is baked into the captured launches
        saved[i] = views[i].ctx->raster_wpsm;
        views[i].ctx->raster_wpsm = (int)cfg.warps_per_sm;
      }
      int r = batch_capture(b, views, n, s, cfg.multi_view == 1, cfg.lane_order, &ex, &nodes);
      for (uint32_t i = 0; i < n; ++i) views[i].ctx->raster_wpsm = saved[i];
      if (r == OIT_OK && !b->raster_pinned) {
        float ms = 0.f;
        r = time_graph(ex, b->stream, 3, &ms);
        if (r == OIT_OK && ms >= best_ms) {
          cudaGraphExecDestroy(ex);
          continue;
        }
        best_ms = ms;
      }
      if (r != OIT_OK) {
        if (ex) cudaGraphExecDestroy(ex);
        if (best) cudaGraphExecDestroy(best);
        return r;
      }
      if (best) cudaGraphExecDestroy(best);
      best = ex;
      best_launches = nodes;
      best_cfg = cfg;
    }
    OIT_TRY_CUDA(cudaStreamSynchronize(b->stream), "sync");
    b->exec = best;
    b->sig = sig;
    b->graph_launches = best_launches;
    b->raster_cfg = best_cfg;
    b->raster_known = true;
    return OIT_OK;  // the plain frames produced this call's images
  }
  for (uint32_t i = 0; i < n; ++i) {  // each view's newest scene constants, before the replay
    const int ur = views[i].ctx->upload_scene(s);
    if (ur != OIT_OK) return ur;
  }
  OIT_TRY_CUDA(cudaEventRecord(b->in, s), "event");
  OIT_TRY_CUDA(cudaStreamWaitEvent(b->stream, b->in, 0), "wait");
  OIT_TRY_CUDA(cudaGraphLaunch(b->exec, b->stream), "graph launch");
  OIT_TRY_CUDA(cudaEventRecord(b->out, b->stream), "event");
  OIT_TRY_CUDA(cudaStreamWaitEvent(s, b->out, 0), "wait");
  for (uint32_t i = 0; i < n; ++i) {
    oit_context* c = b->ctxs[i];
    int r = c->after_graph_launch(b->stream);
    if (r != OIT_OK) return r;
    c->launches += 0;
    c->opaque_valid = b->opaque_valid[i];
    c->color_valid = true;
    c->last_stream = s;
  }
  return OIT_OK;
}

int oit_batch_resolve(oit_batch* b, const oit_view_frame* views, uint32_t n, void* stream) {
  if (!b || !views || n == 0) return OIT_ERR_INVALID_ARGUMENT;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  for (uint32_t i = 0; i < n; ++i) {
    if (!views[i].ctx) return OIT_ERR_INVALID_ARGUMENT;
    if (!views[i].ctx->color_valid) return OIT_ERR_STATE;
    for (uint32_t j = 0; j < i; ++j)
      if (views[j].ctx == views[i].ctx) return OIT_ERR_INVALID_ARGUMENT;
  }
  int r = batch_prepare_resolve(b, views, n);
  if (r != OIT_OK) return r;
  for (uint32_t i = 0; i < n; ++i) {
    oit_context* c = views[i].ctx;
    if (c->batch_resolvable()) continue;
    r = c->composite(views[i].out_rgba8_device, s);
    if (r != OIT_OK) return r;
  }
  uint64_t launches = 0;
  r = b->r_tuned ? batch_resolve_launch(b, s, &launches) : batch_autotune(b, s);
  for (uint32_t i = 0; i < n; ++i) views[i].ctx->last_stream = s;
  return r;
}

int oit_batch_set_resolve_config(oit_batch* b, uint32_t part, const oit_resolve_shape* shape) {
  if (!b || part > 1) return OIT_ERR_INVALID_ARGUMENT;
  oit_batch::Pin pn;
  if (shape) {
    const oit_resolve_shape& sh = *shape;
    if (sh.threads_per_block < 32 || sh.threads_per_block > 256 || sh.threads_per_block % 32 != 0)
      return OIT_ERR_INVALID_ARGUMENT;
    if ((sh.binned != 0 && sh.binned != 1) || (sh.tile_order != 0 && sh.tile_order != 1) ||
        (sh.bin_edges != 0 && sh.bin_edges != 1) ||
        (sh.dense != 0 && sh.dense != 1) || (sh.items_per_step != 0 && sh.items_per_step != 1 && sh.items_per_step != 2))
      return OIT_ERR_INVALID_ARGUMENT;
    const bool x2 = sh.items_per_step == 2;
    if (part == 1) {
      if (sh.shared_slots != 0 || sh.register_slots != 0 || (x2 && sh.dense)) return OIT_ERR_INVALID_ARGUMENT;
      pn.variant = x2 ? oit::kResolveVariantLoop64x2
                      : (sh.dense ? oit::kResolveVariantLoop64Dense : oit::kResolveVariantLoop64);
    } else {
      if ((sh.shared_slots != 0 && sh.shared_slots != 8) ||
          (sh.register_slots != 0 && sh.register_slots != 4 && sh.register_slots != 8))
        return OIT_ERR_INVALID_ARGUMENT;
      if ((sh.shared_slots != 0) + (sh.register_slots != 0) + (int)x2 > 1) return OIT_ERR_INVALID_ARGUMENT;
      if (sh.dense && (sh.shared_slots != 0 || sh.register_slots == 4 || x2)) return OIT_ERR_INVALID_ARGUMENT;
      if (sh.shared_slots) pn.variant = oit::kResolveVariantListShared;
      else if (x2) pn.variant = oit::kResolveVariantListx2;
      else if (sh.register_slots == 4) pn.variant = oit::kResolveVariantListShort4;
      else if (sh.register_slots == 8)
        pn.variant = sh.dense ? oit::kResolveVariantListShort8Dense : oit::kResolveVariantListShort8;
      else pn.variant = sh.dense ? oit::kResolveVariantListDense : oit::kResolveVariantList;
    }
    pn.set = true;
    pn.threads = (int)sh.threads_per_block;
    pn.blocks = (int)std::min<uint32_t>(sh.blocks, 1u << 20);
    pn.binned = sh.binned != 0;
    pn.order = sh.tile_order;
    pn.edges = sh.bin_edges;
  }
  b->pin[part] = pn;
  // tune (or apply the pins) again on the next render or resolve, and capture
  // again; a replay of the old graph may still be running on the batch stream
  if (b->stream) OIT_TRY_CUDA(cudaStreamSynchronize(b->stream), "sync");
  b->r_tuned = false;
  b->drop();
  return OIT_OK;
}

int oit_batch_set_raster_config(oit_batch* b, const oit_raster_config* cfg) {
  if (!b) return OIT_ERR_INVALID_ARGUMENT;
  if (cfg) {
    if (cfg->multi_view != 0 && cfg->multi_view != 1) return OIT_ERR_INVALID_ARGUMENT;
    if (cfg->warps_per_sm != 0 && cfg->warps_per_sm != 32 && cfg->warps_per_sm != 36) return OIT_ERR_INVALID_ARGUMENT;
    if (cfg->multi_view && cfg->warps_per_sm == 32) return OIT_ERR_INVALID_ARGUMENT;
    if (cfg->lane_order != 0 && cfg->lane_order != 1) return OIT_ERR_INVALID_ARGUMENT;
  }
  if (b->stream) OIT_TRY_CUDA(cudaStreamSynchronize(b->stream), "sync");
  b->raster_pinned = cfg != nullptr;
  if (cfg)
    b->raster_pin =
        oit_raster_config{cfg->multi_view, cfg->warps_per_sm == 36 ? 0u : cfg->warps_per_sm, cfg->lane_order};
  b->drop();  // captured again on the next render
  return OIT_OK;
}

int oit_batch_raster_config(oit_batch* b, oit_raster_config* cfg) {
  if (!b || !cfg) return OIT_ERR_INVALID_ARGUMENT;
  if (!b->raster_known) return OIT_ERR_STATE;
  *cfg = b->raster_cfg;
  if (cfg->warps_per_sm == 0) cfg->warps_per_sm = 36;
  return OIT_OK;
}

int oit_batch_resolve_config(oit_batch* b, uint32_t part, oit_resolve_shape* out) {
  if (!b || part > 1 || !out) return OIT_ERR_INVALID_ARGUMENT;
  if (!b->r_tuned) return OIT_ERR_STATE;
  const oit_batch::ResolvePart& rp = b->rparts[part];
  *out = oit_resolve_shape{};
  if (rp.rb.num_views == 0) return OIT_OK;
  out->threads_per_block = (uint32_t)rp.threads;
  out->blocks = (uint32_t)rp.blocks;
  // blocks actually launched when both parts run side by side
  const bool two = b->rparts[0].rb.num_views > 0 && b->rparts[1].rb.num_views > 0 && b->lanes.size() >= 2;
  if (two && b->r_share < 1.0f)
    out->blocks = (uint32_t)std::max(1, (int)((float)rp.blocks * (part == 0 ? b->r_share : 1.0f - b->r_share)));
  out->binned = rp.binned ? 1 : 0;
  out->tile_order = rp.order;
  out->bin_edges = rp.binned ? rp.edges : 0;
  out->shared_slots = rp.variant == oit::kResolveVariantListShared ? 8 : 0;
  out->items_per_step = (rp.variant == oit::kResolveVariantListx2 || rp.variant == oit::kResolveVariantLoop64x2) ? 2 : 1;
  out->register_slots = rp.variant == oit::kResolveVariantListShort4 ? 4
                        : (rp.variant == oit::kResolveVariantListShort8 ||
                           rp.variant == oit::kResolveVariantListShort8Dense)
                            ? 8
                            : 0;
  out->dense = (rp.variant == oit::kResolveVariantListDense || rp.variant == oit::kResolveVariantListShort8Dense ||
                rp.variant == oit::kResolveVariantLoop64Dense)
                   ? 1
                   : 0;
  return OIT_OK;
}

int oit_debug_fail_allocations(int32_t after) {
  if (after < -1) return OIT_ERR_INVALID_ARGUMENT;
  g_fail_alloc_countdown.store(after);
  return OIT_OK;
}

int oit_debug_hold_arrival_lock(oit_context* ctx, int32_t element) {
  if (!ctx || element < -1 || (element >= 0 && (uint64_t)element >= ctx->P)) return OIT_ERR_INVALID_ARGUMENT;
  ctx->debug_held_lock = element;
  ctx->drop_graph();  // a captured frame holds the launch parameters
  return OIT_OK;
}

int oit_get_error(oit_context* ctx, uint32_t* bits) {
  if (!ctx || !bits) return OIT_ERR_INVALID_ARGUMENT;
  OIT_TRY_CUDA(cudaStreamSynchronize(ctx->last_stream), "sync");
  OIT_TRY_CUDA(cudaMemcpy(bits, ctx->err.p, 4, cudaMemcpyDeviceToHost), "d2h");
  OIT_TRY_CUDA(cudaMemset(ctx->err.p, 0, 4), "memset");
  return OIT_OK;
}

int oit_get_buffer(oit_context* ctx, int which, void** ptr, size_t* bytes) {
  if (!ctx || !ptr) return OIT_ERR_INVALID_ARGUMENT;
  DevBuf* b = nullptr;
  size_t n = 0;
  switch (which) {
    case OIT_BUF_ABUFFER: b = &ctx->abuf; n = b->bytes; break;
    case OIT_BUF_AUX: b = &ctx->aux; n = (size_t)ctx->P * ctx->ssn * 4; break;
    case OIT_BUF_AUXDEPTH: b = &ctx->auxdepth; n = (size_t)ctx->P * ctx->ssn * 4; break;
    case OIT_BUF_COUNTER: b = &ctx->counter; n = 4; break;
    case OIT_BUF_DEPTH: b = &ctx->depth; n = ctx->opaque_valid ? (size_t)ctx->S * ctx->P * 4 : 0; break;
    case OIT_BUF_OPAQUE_COLOR: b = &ctx->opaque_color; n = ctx->opaque_valid ? (size_t)ctx->S * ctx->P * 16 : 0; break;
    case OIT_BUF_COLOR: b = &ctx->color; n = (size_t)ctx->P * ctx->ssn * ctx->color_bytes(); break;
    case OIT_BUF_ACCUM: b = &ctx->accum; n = b->bytes; break;
    case OIT_BUF_REVEAL: b = &ctx->reveal; n = b->bytes; break;
    case OIT_BUF_OUTPUT: b = &ctx->out; n = (size_t)ctx->W * ctx->H * 4; break;
    case OIT_BUF_OUTPUT_LINEAR: b = &ctx->out_linear; n = b->p ? (size_t)ctx->W * ctx->H * 16 : 0; break;
    case OIT_BUF_MICROTILE_LENGTHS: b = &ctx->lens; n = b->p ? ctx->lens_count() : 0; break;
    default: return OIT_ERR_INVALID_ARGUMENT;
  }
  *ptr = b->p;
  if (bytes) *bytes = n;
  return OIT_OK;
}

int oit_get_fragment_count(oit_context* ctx, uint64_t* fragments) {
  if (!ctx || !fragments) return OIT_ERR_INVALID_ARGUMENT;
  OIT_TRY_CUDA(cudaStreamSynchronize(ctx->last_stream), "sync");
  unsigned long long v = 0;
  OIT_TRY_CUDA(cudaMemcpy(&v, ctx->frag.p, 8, cudaMemcpyDeviceToHost), "d2h");
  *fragments = v;
  return OIT_OK;
}

int oit_get_launch_count(oit_context* ctx, uint64_t* launches) {
  if (!ctx || !launches) return OIT_ERR_INVALID_ARGUMENT;
  *launches = ctx->launches;
  return OIT_OK;
}

int oit_profile_enable(oit_context* ctx, int enable) {
  if (!ctx) return OIT_ERR_INVALID_ARGUMENT;
  int r = ctx->prof_collect();
  if (r != OIT_OK) return r;
  ctx->prof_on = enable != 0;
  for (int i = 0; i < OIT_PROF_NUM_SECTIONS; ++i) {
    ctx->prof_ms[i] = 0.0;
    ctx->prof_n[i] = 0;
  }
  return OIT_OK;
}

int oit_profile_read(oit_context* ctx, double* total_ms, uint64_t* count) {
  if (!ctx || !total_ms || !count) return OIT_ERR_INVALID_ARGUMENT;
  int r = ctx->prof_collect();
  if (r != OIT_OK) return r;
  for (int i = 0; i < OIT_PROF_NUM_SECTIONS; ++i) {
    total_ms[i] = ctx->prof_ms[i];
    count[i] = ctx->prof_n[i];
  }
  return OIT_OK;
}

const char* oit_status_string(int status) {
  switch (status) {
    case OIT_OK: return "ok";
    case OIT_ERR_INVALID_ARGUMENT: return "invalid argument";
    case OIT_ERR_UNSUPPORTED: return "unsupported configuration";
    case OIT_ERR_OUT_OF_MEMORY: return "out of device memory";
    case OIT_ERR_CUDA: return "CUDA error";
    case OIT_ERR_DEVICE: return "device error flag raised";
    case OIT_ERR_STATE: return "call out of order";
    case OIT_ERR_TOO_LARGE: return "frame exceeds the no-allocation scratch arena";
    default: return "unknown status";
  }
}

}  // extern "C"
