// kernel_abi.cuh — kernel-level launchers on caller-owned device buffers
// (include/onegraph_kernels.h): the engine's relax and gather kernels for a
// caller-built compacted frontier, a check of the bounded device waits, and
// the host-link probe used by the rooflines.  The reference's kernels are
// free functions of this kind: raw device pointers plus a queue
// (bfs_kernelStatic, BFS/oneGraph_BFS/gpu_kernels.h:211-241; sssp_kernel,
// SSSP/oneGraph/gpu_kernels.h:177-203; cc_kernelStaticSwap,
// CC/onegraph/gpu_kernels.h:133-157).
// A section of the engine's translation unit (engine.cu includes it after
// its own launchers), so the header-defined kernels are compiled once.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/onegraph_kernels.h"
#include "batch_persist.cuh"
#include "kernels.cuh"
#include "og_internal.hpp"

namespace kabi {

using namespace og;

constexpr int kGatherMultAbi = 2;  // gather tiles of 4096 positions, as in the engine

// Error word on the device for one launch; released by the destructor.
struct ErrWord {
  uint32_t *d = nullptr;
  ~ErrWord() {
    if (d) cudaFree(d);
  }
};

int finish(cudaStream_t s, ErrWord &w, const char *what) {
  uint32_t err = 0;
  cudaError_t ce = cudaGetLastError();
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&err, w.d, 4, cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return fail(OG_E_CUDA, "%s: %s", what, cudaGetErrorString(ce));
  if (err & (kErrLookback | kErrBarrier)) return fail(OG_E_TIMEOUT, "%s: a bounded wait gave up", what);
  if (err) return fail(OG_E_DEVICE, "%s: out-of-range index (flags 0x%x)", what, err);
  return OG_OK;
}

int list_args_ok(const uint32_t *list, const uint64_t *pref, const uint32_t *tile, uint64_t total,
                 const uint64_t *off, const og_k_records *rec) {
  if (!list || !pref || !tile || !off || !rec || !rec->words) return fail(OG_E_ARG, "null argument");
  if (rec->bpe == 0 || rec->bpe > 64 || rec->bc == 0 || rec->bc > rec->bpe || rec->bc > 32)
    return fail(OG_E_ARG, "bad record layout (bpe %u, bc %u)", rec->bpe, rec->bc);
  if (total / kTile > 0x7fffffffull) return fail(OG_E_ARG, "list too long");
  return OG_OK;
}

LbsArgs lbs_for(const uint32_t *list, const uint64_t *pref, const uint32_t *tile, uint32_t n, uint64_t total,
                const uint64_t *off, const og_k_records *rec, uint64_t pb, uint64_t pe, uint32_t *err) {
  LbsArgs a;
  a.list = list;
  a.pref = pref;
  a.tile_first = tile;
  a.n = n;
  a.total = total;
  a.pos_begin = pb;
  a.pos_end = pe;
  a.off = off;
  a.stage_base = pb;
  a.edge_bound = rec->nrecords;
  a.err = err;
  return a;
}

__global__ void k_wait_check(int which, uint32_t spin_limit, uint32_t *scratch, uint32_t *err) {
  if (which == 0) {
    // tile 1 of a compaction whose tile 0 never publishes (its status word
    // stays 0, never this launch's epoch 1)
    if (threadIdx.x >= 32) return;
    Lookback lb;
    lb.status = scratch;
    lb.ticket = scratch + 2;
    lb.agg_n = scratch + 4;
    lb.inc_n = scratch + 8;
    lb.agg_e = (unsigned long long *)(scratch + 16);
    lb.inc_e = (unsigned long long *)(scratch + 24);
    uint32_t pn;
    uint64_t pe;
    int bad;
    lookback_prefix(lb, 1, 1, 0, 0, err, pn, pe, bad, spin_limit);
  } else {
    // a barrier expecting one CTA more than the launch holds
    grid_barrier((unsigned int *)scratch, err, gridDim.x + 1, spin_limit);
  }
}

// Streams `words` 16-byte words of page-locked host memory through the SMs
// (coalesced, grid-stride, every load feeding an XOR so none is dropped).
__global__ void __launch_bounds__(256) k_link_read(const uint4 *src, uint64_t words, uint32_t *sink) {
  uint32_t acc = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  for (; i + 3 * stride < words; i += 4 * stride) {  // four loads in flight per thread
    const uint4 a = __ldcv(src + i), b = __ldcv(src + i + stride), c = __ldcv(src + i + 2 * stride),
                d = __ldcv(src + i + 3 * stride);
    acc ^= a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w ^ c.x ^ c.y ^ c.z ^ c.w ^ d.x ^ d.y ^ d.z ^ d.w;
  }
  for (; i < words; i += stride) {
    const uint4 a = __ldcv(src + i);
    acc ^= a.x ^ a.y ^ a.z ^ a.w;
  }
  if (acc == 0x9e3779b9u) atomicAdd(sink, 1u);  // data-dependent: the loads stay
}

}  // namespace kabi

using namespace kabi;

extern "C" int og_k_relax(int algo, const uint32_t *list, const uint64_t *pref, const uint32_t *tile,
                          uint32_t n, uint64_t total, const uint64_t *off, const og_k_records *rec,
                          uint32_t V, uint32_t *value, uint32_t *next, uint32_t *visited, uint32_t level,
                          void *stream) {
  clear_error();
  int rc = list_args_ok(list, pref, tile, total, off, rec);
  if (rc != OG_OK) return rc;
  if (!value || !next || (algo == OG_ALGO_BFS && !visited)) return fail(OG_E_ARG, "null value or bitmap");
  if (algo != OG_ALGO_BFS && algo != OG_ALGO_SSSP && algo != OG_ALGO_CC)
    return fail(OG_E_ARG, "og_k_relax: algorithm %d", algo);
  cudaGetLastError();
  cudaStream_t s = (cudaStream_t)stream;
  ErrWord w;
  CK(cudaMalloc(&w.d, 4));
  CK(cudaMemsetAsync(w.d, 0, 4, s));
  const unsigned grid = (unsigned)((total + kTile - 1) / kTile);
  if (n && grid) {
    const LbsArgs a = lbs_for(list, pref, tile, n, total, off, rec, 0, total, w.d);
    if (algo == OG_ALGO_BFS) {
      BfsOp op{visited, next, value, w.d, V, level + 1};
      k_lbs<SrcP<false>, BfsOp><<<grid, kThreads, 0, s>>>(a, SrcP<false>{rec->words, rec->bpe, rec->bc, rec->wmin}, op);
    } else if (algo == OG_ALGO_SSSP) {
      MinOp<true> op{value, next, w.d, V};
      k_lbs<SrcP<true>, MinOp<true>><<<grid, kThreads, 0, s>>>(a, SrcP<true>{rec->words, rec->bpe, rec->bc, rec->wmin},
                                                               op);
    } else {
      MinOp<false> op{value, next, w.d, V};
      k_lbs<SrcP<false>, MinOp<false>><<<grid, kThreads, 0, s>>>(a, SrcP<false>{rec->words, rec->bpe, rec->bc, rec->wmin},
                                                                 op);
    }
  }
  return finish(s, w, "og_k_relax");
}

extern "C" int og_k_gather(const uint32_t *list, const uint64_t *pref, const uint32_t *tile, uint32_t n,
                           uint64_t total, const uint64_t *off, const og_k_records *rec, uint64_t pos_begin,
                           uint64_t pos_end, uint32_t *out_col, uint32_t *out_w, void *stream) {
  clear_error();
  int rc = list_args_ok(list, pref, tile, total, off, rec);
  if (rc != OG_OK) return rc;
  if (!out_col) return fail(OG_E_ARG, "null output");
  // the kernel finds a tile's last vertex through the tile map, so a range
  // ends on a tile boundary or at the end of the list, as the engine's
  // staging chunks do
  if (pos_begin % kTile || pos_begin > pos_end || pos_end > total || (pos_end % kTile && pos_end != total))
    return fail(OG_E_ARG, "positions [%llu, %llu) of %llu (both ends multiples of %u, or the end = total)",
                (unsigned long long)pos_begin, (unsigned long long)pos_end, (unsigned long long)total, kTile);
  cudaGetLastError();
  cudaStream_t s = (cudaStream_t)stream;
  ErrWord w;
  CK(cudaMalloc(&w.d, 4));
  CK(cudaMemsetAsync(w.d, 0, 4, s));
  constexpr uint64_t T = (uint64_t)kGatherMultAbi * kTile;
  const unsigned grid = (unsigned)((pos_end - pos_begin + T - 1) / T);
  const int smem = (int)gather_smem_bytes<kGatherMultAbi>();
  if (n && grid) {
    const LbsArgs a = lbs_for(list, pref, tile, n, total, off, rec, pos_begin, pos_end, w.d);
    if (out_w) {
      auto k = k_gather<SrcP<true>, DstW<uint32_t>, kGatherMultAbi>;
      CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      k<<<grid, kThreads, smem, s>>>(a, SrcP<true>{rec->words, rec->bpe, rec->bc, rec->wmin},
                                     DstW<uint32_t>{out_col, out_w});
    } else {
      auto k = k_gather<SrcP<false>, DstU, kGatherMultAbi>;
      CK(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      k<<<grid, kThreads, smem, s>>>(a, SrcP<false>{rec->words, rec->bpe, rec->bc, rec->wmin}, DstU{out_col});
    }
  }
  return finish(s, w, "og_k_gather");
}

extern "C" int og_k_wait_check(int which, uint32_t spin_limit) {
  clear_error();
  if (which != 0 && which != 1) return fail(OG_E_ARG, "og_k_wait_check: which = %d", which);
  cudaGetLastError();
  ErrWord w;
  uint32_t *scratch = nullptr;
  CK(cudaMalloc(&w.d, 4));
  if (cudaMalloc(&scratch, 256) != cudaSuccess) return fail(OG_E_CUDA, "og_k_wait_check: cudaMalloc");
  struct Free {
    uint32_t *p;
    ~Free() { cudaFree(p); }
  } free_scratch{scratch};
  CK(cudaMemset(w.d, 0, 4));
  CK(cudaMemset(scratch, 0, 256));
  k_wait_check<<<1, which == 0 ? 32 : kThreads>>>(which, spin_limit, scratch, w.d);
  return finish(nullptr, w, which == 0 ? "compaction look-back" : "grid barrier");
}

extern "C" int og_link_probe(const void *host, uint64_t bytes, int mode, int reps, double *gbs) {
  clear_error();
  if (!host || !gbs || bytes < (1u << 20) || bytes % 16 || reps < 1 || mode < 0 || mode > 2)
    return fail(OG_E_ARG, "og_link_probe: bad argument");
  cudaGetLastError();
  cudaPointerAttributes pa;
  CK(cudaPointerGetAttributes(&pa, host));
  if (pa.type != cudaMemoryTypeHost) return fail(OG_E_ARG, "og_link_probe: buffer is not page-locked host memory");
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  cudaStream_t s[2] = {nullptr, nullptr};
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  void *dbuf = nullptr;
  uint32_t *sink = nullptr;
  struct Cleanup {
    cudaStream_t *s;
    cudaEvent_t *ev;
    void **d;
    uint32_t **k;
    ~Cleanup() {
      for (int i = 0; i < 2; i++)
        if (s[i]) cudaStreamDestroy(s[i]);
      for (int i = 0; i < 4; i++)
        if (ev[i]) cudaEventDestroy(ev[i]);
      if (*d) cudaFree(*d);
      if (*k) cudaFree(*k);
    }
  } cleanup{s, ev, &dbuf, &sink};
  for (int i = 0; i < 2; i++) CK(cudaStreamCreateWithFlags(&s[i], cudaStreamNonBlocking));
  for (int i = 0; i < 4; i++) CK(cudaEventCreate(&ev[i]));
  CK(cudaMalloc(&sink, 4));
  const void *dview = nullptr;
  if (mode == 0) {
    CK(cudaHostGetDevicePointer((void **)&dview, const_cast<void *>(host), 0));
  } else {
    CK(cudaMalloc(&dbuf, bytes));
  }
  double best = 0;
  for (int r = 0; r <= reps; r++) {  // the first run is a warm-up
    CK(cudaEventRecord(ev[0], s[0]));
    if (mode == 0) {
      k_link_read<<<(unsigned)sms * 8, 256, 0, s[0]>>>((const uint4 *)dview, bytes / 16, sink);
      CK(cudaGetLastError());
    } else if (mode == 1) {
      CK(cudaMemcpyAsync(dbuf, host, bytes, cudaMemcpyHostToDevice, s[0]));
    } else {
      const uint64_t half = bytes / 32 * 16;
      CK(cudaStreamWaitEvent(s[1], ev[0], 0));
      CK(cudaMemcpyAsync(dbuf, host, half, cudaMemcpyHostToDevice, s[0]));
      CK(cudaMemcpyAsync((char *)dbuf + half, (const char *)host + half, bytes - half, cudaMemcpyHostToDevice,
                         s[1]));
      CK(cudaEventRecord(ev[2], s[1]));
      CK(cudaStreamWaitEvent(s[0], ev[2], 0));
    }
    CK(cudaEventRecord(ev[1], s[0]));
    CK(cudaEventSynchronize(ev[1]));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    if (r > 0 && ms > 0) best = std::max(best, bytes / (ms / 1e3) / 1e9);
  }
  *gbs = best;
  return OG_OK;
}
