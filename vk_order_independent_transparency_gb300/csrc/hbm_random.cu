// HBM throughput for the access patterns of the resolve: a sequential read,
// independent random reads of G contiguous bytes (G-aligned, a warp's 32
// reads inside one window of the buffer), and dependent chains of 16-byte
// reads (each offset comes from the previous read, like a linked-list walk).
// Prints one JSON object. A measurement program run by bench.py --hbm-random;
// not part of the library.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <type_traits>

namespace {

__device__ __forceinline__ uint32_t h32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__global__ void k_seq(const uint4* __restrict__ buf, uint64_t n16, uint32_t* out) {
  uint32_t acc = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 v = __ldg(buf + i);
    acc += v.x ^ v.w;
  }
  if (acc == 0x12345678u) out[0] = acc;
}

// slot s of window w: (w << wlog) | s, G bytes each; every index < nwin << wlog
template <int G>
__global__ void k_random(const uint4* __restrict__ buf, uint32_t nwin_mask, int wlog, uint32_t n, uint32_t* out) {
  uint32_t acc = 0;
  const uint32_t smask = (1u << wlog) - 1u;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint64_t slot = ((uint64_t)(h32(i >> 5) & nwin_mask) << wlog) | (h32(i * 2654435761u) & smask);
    const uint4* p = buf + slot * (G / 16);
#pragma unroll
    for (int k = 0; k < G / 16; ++k) {
      const uint4 v = __ldg(p + k);
      acc += v.x ^ v.w;
    }
  }
  if (acc == 0x12345678u) out[0] = acc;
}

__global__ void k_chain(const uint4* __restrict__ buf, uint32_t nwin_mask, int wlog, int steps, uint32_t* out) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t smask = (1u << wlog) - 1u;
  const uint64_t base = (uint64_t)(h32(t >> 5) & nwin_mask) << wlog;
  uint32_t s = h32(t) & smask, acc = 0;
  for (int j = 0; j < steps; ++j) {
    const uint4 v = __ldg(buf + base + s);
    acc += v.x;
    s = h32(s ^ v.x) & smask;  // the buffer holds zeros: the next offset waits for this read
  }
  if (acc == 0x12345678u) out[0] = acc;
}

int lg2(uint64_t v) {
  int r = 0;
  while ((1ull << r) < v) ++r;
  return r;
}

}  // namespace

int main() {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess) return 1;
  const uint64_t bytes = 4ull << 30;
  uint4* buf = nullptr;
  uint32_t* out = nullptr;
  if (cudaMalloc(&buf, bytes) != cudaSuccess || cudaMalloc(&out, 4) != cudaSuccess) return 1;
  cudaMemset(buf, 0, bytes);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float ms = 0.f;
  auto timed = [&](auto launch) {
    launch();  // warm-up
    cudaEventRecord(a);
    launch();
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&ms, a, b);
    return ms;
  };
  printf("{\"buffer_bytes\": %llu, \"sequential_read_gbs\": %.1f", (unsigned long long)bytes,
         bytes / timed([&] { k_seq<<<sms * 8, 256>>>(buf, bytes / 16, out); }) / 1e6);
  const uint32_t n = 256u << 20;  // reads per measurement
  printf(", \"random_read_gbs\": {");
  bool first = true;
  for (uint64_t win_mb : {32ull, 256ull, 4096ull}) {
    const uint32_t nwin_mask = (uint32_t)(bytes / (win_mb << 20)) - 1u;
    auto one = [&](auto g) {
      constexpr int G = decltype(g)::value;
      const int wlog = lg2((win_mb << 20) / G);
      const float t = timed([&] { k_random<G><<<sms * 8, 256>>>(buf, nwin_mask, wlog, n, out); });
      printf("%s\"G%d_window%lluMB\": %.1f", first ? "" : ", ", G, (unsigned long long)win_mb, (double)n * G / t / 1e6);
      first = false;
    };
    one(std::integral_constant<int, 16>{});
    one(std::integral_constant<int, 32>{});
    one(std::integral_constant<int, 64>{});
  }
  printf("}, \"chain16_gbs\": {");
  first = true;
  for (uint64_t win_mb : {32ull, 256ull, 4096ull}) {
    const uint32_t nwin_mask = (uint32_t)(bytes / (win_mb << 20)) - 1u;
    const int wlog = lg2((win_mb << 20) / 16);
    const int blocks = sms * 8, threads = 256, steps = 64;  // 64 warps per SM
    const float t = timed([&] { k_chain<<<blocks, threads>>>(buf, nwin_mask, wlog, steps, out); });
    printf("%s\"window%lluMB\": %.1f", first ? "" : ", ", (unsigned long long)win_mb,
           (double)blocks * threads * steps * 16 / t / 1e6);
    first = false;
  }
  const cudaError_t e = cudaDeviceSynchronize();
  printf("}, \"status\": \"%s\"}\n", cudaGetErrorString(e));
  cudaFree(buf);
  cudaFree(out);
  return e == cudaSuccess ? 0 : 2;
}
