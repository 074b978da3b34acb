// probe.cu — the measured load bandwidth of the L1 data cache, the
// denominator of the marchers' roofline.
//
// The marchers read cache-resident tables (volume quads, SAT quads, pyramid
// quads) with 16-byte gathers: their bound is the L1/TEX load path, not HBM.
// k_l1_probe streams coalesced 16-byte non-coherent loads (the marchers'
// load instruction) over a 16 KB buffer that every SM keeps in its L1, so its
// rate is the L1 hit bandwidth of that instruction on this part.
#include <algorithm>

#include <cuda_runtime.h>

#include "ctx.cuh"

namespace {

constexpr int kProbeEntries = 1024;  // 16 KB of uint4
constexpr int kProbeThreads = 512;
constexpr int kProbeUnroll = 8;

__global__ void __launch_bounds__(kProbeThreads) k_l1_probe(const uint4* __restrict__ buf, int iters,
                                                            unsigned* __restrict__ sink) {
  uint4 acc = make_uint4(0, 0, 0, 0);
  // warp w reads 32 consecutive entries (512 contiguous bytes) per load;
  // the window moves by one warp-width per load so no load can be hoisted
  const unsigned lane0 = threadIdx.x;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kProbeUnroll; ++k) {
      const unsigned i = (lane0 + (unsigned)(it * kProbeUnroll + k) * 32u) & (kProbeEntries - 1);
      const uint4 v = __ldg(buf + i);
      acc.x ^= v.x; acc.y ^= v.y; acc.z ^= v.z; acc.w ^= v.w;
    }
  }
  if ((acc.x ^ acc.y ^ acc.z ^ acc.w) == 0x9E3779B9u) sink[0] = acc.x;  // keeps the loads live
}

}  // namespace

extern "C" cvr_status cvr_measure_l1_bandwidth(cvr_ctx* c, float* gbs) {
  using namespace cvr::ctxutil;
  if (!c || !gbs) return CVR_ERR_INVALID_ARG;
  CK(c, cudaSetDevice(c->device));
  int sms = 0;
  CK(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  uint4* buf = nullptr;
  CK(c, ensure(c->d_probe, c->probe_cap, kProbeEntries * sizeof(uint4) + 256));
  buf = reinterpret_cast<uint4*>(c->d_probe);
  CK(c, launch_fill(buf, kProbeEntries * sizeof(uint4), 0x01234567u, c->stream));
  unsigned* sink = reinterpret_cast<unsigned*>(reinterpret_cast<char*>(c->d_probe) + kProbeEntries * sizeof(uint4));
  const int blocks = sms * 4, iters = 1024;
  k_l1_probe<<<blocks, kProbeThreads, 0, c->stream>>>(buf, iters, sink);  // warm-up (fills every L1)
  CK(c, cudaGetLastError());
  float best = 0.0f;
  for (int rep = 0; rep < 5; ++rep) {
    CK(c, cudaEventRecord(c->ev[0], c->stream));
    k_l1_probe<<<blocks, kProbeThreads, 0, c->stream>>>(buf, iters, sink);
    CK(c, cudaEventRecord(c->ev[1], c->stream));
    CK(c, cudaEventSynchronize(c->ev[1]));
    float ms = 0.0f;
    CK(c, cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
    const double bytes = (double)blocks * kProbeThreads * iters * kProbeUnroll * sizeof(uint4);
    best = std::max(best, (float)(bytes / (ms * 1e-3) / 1e9));
  }
  *gbs = best;
  return CVR_OK;
}
