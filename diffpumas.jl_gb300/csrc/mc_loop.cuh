// mc_loop.cuh -- the persistent history loop shared by the backward MC
// kernels (two-layer geometry in mc.cu, fixed directional paths in
// dir_mc.cu): table staging, history hand-out, the phase hand-off queue and
// the warp-cooperative evaluation of hard-event DCS sums.
//
// A geometry G supplies the history type and its transport:
//   G::Hist, G::Queue                         history state, hand-off record
//   long n0() const                           histories of phase 0
//   void start(long i, Hist&, Stream&)        history i from its start record
//   long load(const Queue&, Hist&, Stream&)   a handed-over history (phase 1)
//   void save(const Hist&, const Stream&, long i, Queue*)
//   void end(long i, const Hist&)             end record of history i
//   const Med<R>& medium(int k) const         medium of a suspended step
//   const Med<R>* media() const               the descriptors by medium index
//   int advance<COOP, PHASE>(Hist&, Stream&)  one step: ADV_*
//   int resume<PHASE>(Hist&, Stream&)         finish a suspended step: ADV_*
#pragma once
#include <cooperative_groups.h>

#include <algorithm>
#include <type_traits>

#include "mc_device.cuh"

namespace dp {
namespace mc {

// Launch shape per precision: one CTA per SM whose warps share one staged
// copy of the tables.  The FP32 transport evaluates hard-event DCS sums
// cooperatively per warp; it is compiled for three CTA sizes that trade
// registers per thread for warps per SM (1024: at most 64 registers, 32
// warps; 768: at most 80, 24 warps; 512: 116, 16 warps), chosen per context
// (dp_set_mc_threads, dp_autotune).  The transport is latency bound, so the
// most warps win: 1024 threads run the two-layer and fixed-path workloads
// 1.3-1.4x faster than 512, with 164 bytes of spills.  The FP64 transport
// (one thread per sum, 255 registers) runs 8 warps.
template <class R> struct KCfg;
template <> struct KCfg<float> {
  static constexpr int threads = 1024;  // default CTA size
  static constexpr bool coop = true;
};
template <> struct KCfg<double> {
  static constexpr int threads = 256;
  static constexpr bool coop = false;
};

// Calls f(std::integral_constant<int, T>{}) with T the compiled CTA size
// matching `threads` (0 or an unknown size: the default).
template <class R, class F>
inline int with_threads(int threads, F&& f) {
  if constexpr (sizeof(R) == 4) {
    if (threads == 768) return f(std::integral_constant<int, 768>{});
    if (threads == 512) return f(std::integral_constant<int, 512>{});
    return f(std::integral_constant<int, 1024>{});
  } else {
    (void)threads;
    return f(std::integral_constant<int, 256>{});
  }
}

// Shared-memory carve-out steps of an SM (KB; the L1 cache gets the rest of
// its 256 KB).  carveout_cap(need): the largest dynamic shared memory of a
// one-CTA launch within the smallest step that holds `need` bytes (1 KB of
// each step is reserved per CTA).  The MC kernels size their DCS buffers to
// it: their 64-register threads spill, and a larger L1 keeps the stack out
// of L2 (c2 53.2 -> 48.5 ms, c4 408 -> 390 ms against filling the SM's
// shared memory).
inline size_t carveout_cap(size_t need) {
  static const int steps[] = {0, 8, 16, 32, 64, 100, 132, 164, 196, 228};
  for (int s : steps)
    if (size_t(s) * 1024 >= need + 1024) return size_t(s) * 1024 - 1024;
  return need;
}
// The carve-out preference (percent of the SM's shared memory) of a kernel
// with `smem` bytes of dynamic shared memory: rounded down, the driver then
// takes the next step that fits.
inline int carveout_percent(int device, size_t smem) {
  int sm_max = 0;
  if (cudaDeviceGetAttribute(&sm_max, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device) !=
          cudaSuccess ||
      sm_max <= 0)
    return -1;  // no preference
  const int pct = int(100.0 * double(smem + 1024) / double(sm_max));
  return pct < 0 ? 0 : (pct > 100 ? 100 : pct);
}

// Events a warp's batched DCS pass serves at once: as many as `avail` bytes of
// shared memory hold for `warps` warps, between 1 and 32 (a warp's lanes).
inline int coop_kmax(size_t avail, int warps, int nel) {
  for (int k = 32; k > 1; --k)
    if (size_t(warps) * size_t(coop_floats(nel, k)) * sizeof(float) <= avail) return k;
  return 1;
}

// Copies `bytes` (16-byte multiple) from global to shared memory with
// cp.async.bulk completing on one mbarrier; all threads call it.  Returns
// false if the wait exceeded `wait_iters` polls (stage_settle has then waited
// for the copy in flight).
static __device__ __noinline__ bool stage_blob(unsigned char* dst, const unsigned char* src, uint32_t bytes,
                                        uint64_t* mbar, int wait_iters) {
  uint32_t bar = smem_u32(mbar);
  mbar_init(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
    const uint32_t chunk = 32768;
    for (uint32_t off = 0; off < bytes; off += chunk) {
      uint32_t b = bytes - off < chunk ? bytes - off : chunk;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              smem_u32(dst + off)),
          "l"(src + off), "r"(b), "r"(bar)
          : "memory");
    }
  }
  return stage_settle(bar, mbar_wait(bar, wait_iters));
}

// Next history index for the calling thread (warp-aggregated atomic).
__device__ __forceinline__ long next_history(unsigned long long* counter) {
  namespace cg = cooperative_groups;
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned long long base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, (unsigned long long)g.size());
  base = g.shfl(base, 0);
  return long(base + g.thread_rank());
}

// A block whose table staging gave up takes its share of the phase's
// histories all the same and ends each one flagged DP_ST_TABLE_WAIT (no flux,
// no table read), so that every history of the launch is accounted for.
template <class R, int PHASE, class G>
__device__ __forceinline__ void drain_histories(G& geo, unsigned long long* counter,
                                                typename G::Queue* queue,
                                                const uint32_t* order = nullptr) {
  const long n = PHASE == 0 ? geo.n0() : long(*(volatile unsigned long long*)(counter + 2));
  typename G::Hist h;
  Stream g;
  for (;;) {
    const long j = next_history(counter + PHASE);
    if (j >= n) break;
    const long k = order ? long(order[j]) : j;
    long i = k;
    if (PHASE == 0) geo.start(k, h, g);
    else i = geo.load(queue[k], h, g);
    h.s.status |= ST_TABLE;
    geo.end(i, h);
  }
}

// CTA form of the batched DCS sums for the lockstep phases.  The buffer at
// `base` (cta_floats(nel, kc) floats) holds two event counters, then for kc
// events: items and components in rows of nel elements (the largest element
// count of the launch's media), totals, ancestor energies, transfers and
// media.  Terms, components and totals come from the helpers coop_batch uses
// (coop_pair, coop_photo, coop_bi, coop_comp, coop_total), in the same order
// per event, so an event's sum does not depend on the events served with it.
// The two forms are compiled apart, and the code generator may fuse their
// FP32 multiply-adds differently.
__host__ __device__ inline int cta_floats(int nel, int kc) {
  return 4 + kc * ((kItemsPerElement + 4) * nel + 4);
}
// Events per chunk of a CTA buffer of `floats` floats (at most `threads`).
inline int cta_kc(int floats, int nel, int threads) {
  int kc = (floats - 4) / ((kItemsPerElement + 4) * nel + 4);
  return kc < threads ? (kc > 0 ? kc : 0) : threads;
}
// meds: the launch's media descriptors, indexed by medium.  (Inlined: out of
// line it shrinks the stack frame by 64 B but the c2 and c4 steps run 3-4%
// slower.)
__device__ __forceinline__ void cta_batch(const Med<float>* meds, float fm, int k, int nel,
                                          float* item, float* comp, float* tot, const float* anc,
                                          const float* q, const int* med) {
  const int t = threadIdx.x, T = blockDim.x;
  const int ni = kItemsPerElement * nel, nc = 4 * nel;
  for (int f = t; f < k * nel * 12; f += T) {
    const int i = f / (nel * 12), r = f - i * nel * 12, e = r / 12, p = r - e * 12;
    const Med<float>& m = meds[med[i]];
    if (e < m.nel)
      item[i * ni + e * kItemsPerElement + 1 + p] = coop_pair(m.elf + kElfStride * e, fm, anc[i], q[i], p);
  }
  for (int f = t; f < k * nel * 9; f += T) {
    const int i = f / (nel * 9), r = f - i * nel * 9, e = r / 9, p = r - e * 9;
    const Med<float>& m = meds[med[i]];
    if (e < m.nel)
      item[i * ni + e * kItemsPerElement + 13 + p] = coop_photo(m.elf + kElfStride * e, fm, anc[i], q[i], p);
  }
  for (int f = t; f < k * nel * 2; f += T) {
    const int i = f / (nel * 2), r = f - i * nel * 2, e = r >> 1, u = r & 1;
    const Med<float>& m = meds[med[i]];
    if (e < m.nel)
      item[i * ni + e * kItemsPerElement + (u ? 22 : 0)] = coop_bi(m.elf + kElfStride * e, fm, anc[i], q[i], u);
  }
  __syncthreads();
  for (int f = t; f < k * nc; f += T) {
    const int i = f / nc, c = f - i * nc, e = c >> 2, p = c & 3;
    const Med<float>& m = meds[med[i]];
    if (e < m.nel)
      comp[i * nc + c] = coop_comp(item + i * ni + e * kItemsPerElement, p, m.elf[kElfStride * e + 3], anc[i]);
  }
  __syncthreads();
  const int lane = t & 31;
  for (int i = t >> 5; i < k; i += T >> 5) {
    const float v = coop_total(comp + i * nc, 4 * meds[med[i]].nel, lane);
    if (lane == 0) tot[i] = v;
  }
  __syncthreads();
}
// Serves every suspended step of the CTA (waits: this thread's step waits on
// a DCS sum; x its continuation) in chunks of kc events; counter `parity` of
// the buffer numbers the events (any numbering gives the same results).
// All threads of the CTA call it.
template <class G, class R>
__device__ __forceinline__ void serve_cta(const G& geo, const Consts& C, float* base, int kc, int nel,
                                          int parity, bool waits, Cont<R>& x, Stream& g) {
  int* cnt = reinterpret_cast<int*>(base) + parity;
  const int ni = kItemsPerElement * nel, nc = 4 * nel;
  float* item = base + 4;
  float* comp = item + kc * ni;
  float* tot = comp + kc * nc;
  float* anc = tot + kc;
  float* q = anc + kc;
  int* med = reinterpret_cast<int*>(q + kc);
  int slot = -1;
  if (waits) {
    namespace cg = cooperative_groups;
    cg::coalesced_group grp = cg::coalesced_threads();
    int b = 0;
    if (grp.thread_rank() == 0) b = atomicAdd(cnt, int(grp.size()));
    slot = grp.shfl(b, 0) + int(grp.thread_rank());
  }
  __syncthreads();
  const int nw = *reinterpret_cast<volatile int*>(cnt);
  for (int c0 = 0; c0 < nw; c0 += kc) {
    const int k = nw - c0 < kc ? nw - c0 : kc;
    const int s = slot - c0;
    const bool mine = slot >= c0 && s < k;
    if (mine) {
      anc[s] = x.anc;
      q[s] = x.q;
      med[s] = x.medium;
    }
    __syncthreads();
    cta_batch(geo.media(), C.mass_f, k, nel, item, comp, tot, anc, q, med);
    if (mine) {
      const int last = 4 * geo.medium(x.medium).nel - 1;
      const float* cp = comp + s * nc;
      const float total = tot[s];
      x.total = total;
      x.pick = -1;
      if (x.details && total > 0.f) {
        // process and element pick in the reference's order (src/MixedTransport.jl:131-140)
        float u = uni<float>(g) * total;
        int pick = last;
        for (int c = 0; c <= last; ++c) {
          u -= cp[c];
          if (u <= 0.f) {
            pick = c;
            break;
          }
        }
        x.pick = pick;
      }
    }
    __syncthreads();  // the next chunk reuses the buffer
  }
}

// Runs histories until none is left for this phase.  counter[PHASE] hands out
// history indices, counter[2] counts the hand-off queue.  With COOP, `coop`
// is the CTA's shared memory for batched DCS sums: per warp `stride` floats
// (coop_floats for up to kmax events of one medium), or, in lockstep, one
// CTA buffer (cta_floats(nel, kc)).  `order` (may be null) maps the j-th
// hand-out to a history (phase 0) or a queue slot (phase 1): the
// longest-first schedule.  With `lockstep` (block-uniform) every warp of the
// CTA runs its loop iterations in step with the others until the CTA has no
// history left, and the CTA serves all its waiting steps together.
template <class R, int PHASE, bool COOP, class G>
__device__ __forceinline__ void transport_histories(G& geo, const Consts& C,
                                                    unsigned long long* counter,
                                                    typename G::Queue* queue, float* coop,
                                                    int stride, int kmax, int kc, int nel,
                                                    const uint32_t* order = nullptr,
                                                    bool lockstep = false) {
  const long n = PHASE == 0 ? geo.n0() : long(*(volatile unsigned long long*)(counter + 2));
  typename G::Hist h;
  Stream g;
  auto take = [&](long* idx) -> bool {
    const long j = next_history(counter + PHASE);
    if (j >= n) return false;
    const long k = order ? long(order[j]) : j;
    if (PHASE == 0) {
      *idx = k;
      geo.start(k, h, g);
    } else {
      *idx = geo.load(queue[k], h, g);
    }
    return true;
  };
  // after a step: end the history, hand it to phase 1, or keep going
  auto settle = [&](int r, long* idx) -> bool {
    if (r == ADV_HANDOFF) {
      unsigned long long slot = atomicAdd(counter + 2, 1ull);
      geo.save(h, g, *idx, queue + slot);
      return take(idx);
    }
    if (r == ADV_DONE) {
      geo.end(*idx, h);
      return take(idx);
    }
    return true;
  };
  long i = 0;
  bool live = take(&i);
  if constexpr (COOP) {
    if (lockstep && kc > 0) {
      int* cnt = reinterpret_cast<int*>(coop);
      if (threadIdx.x == 0) cnt[0] = cnt[1] = 0;
      __syncthreads();
      for (int parity = 0;; parity ^= 1) {
        // counter parity ^ 1 was last read before the previous iteration's barrier
        if (threadIdx.x == 0) cnt[parity ^ 1] = 0;
        serve_cta(geo, C, coop, kc, nel, parity, live && h.x.kind != CONT_NONE, h.x, g);
        if (live) {
          const int r = h.x.kind != CONT_NONE ? geo.template resume<PHASE>(h, g)
                                              : geo.template advance<true, PHASE>(h, g);
          live = settle(r, &i);
        }
        if (!__syncthreads_or(live)) break;
      }
      return;
    }
    const int lane = threadIdx.x & 31;
    coop += size_t(threadIdx.x >> 5) * stride;
    for (;;) {
      // serve the hard events the warp's suspended steps wait for: the
      // waiting lanes of one medium together, up to kmax at a time
      const bool waits = live && h.x.kind != CONT_NONE;
      unsigned want = __ballot_sync(0xffffffffu, waits);
      while (want) {
        const int med = __shfl_sync(0xffffffffu, h.x.medium, __ffs(want) - 1);
        unsigned batch = __ballot_sync(0xffffffffu, ((want >> lane) & 1u) && h.x.medium == med);
        while (__popc(batch) > kmax) batch &= ~(1u << (31 - __clz(batch)));
        want &= ~batch;
        const bool mine = (batch >> lane) & 1u;
        const int slot = __popc(batch & ((1u << lane) - 1u));
        const int k = __popc(batch);
        const Med<R>& m = geo.medium(med);
        float* anc = coop + coop_head(m.nel, k);
        if (mine) {
          anc[slot] = h.x.anc;
          anc[k + slot] = h.x.q;
        }
        __syncwarp();
        coop_batch(m.elf, m.nel, C.mass_f, k, coop);
        if (mine) {
          const int ni = kItemsPerElement * m.nel, nc = 4 * m.nel;
          const float* comp = coop + k * ni + slot * nc;
          const float total = coop[k * ni + k * nc + slot];
          h.x.total = total;
          h.x.pick = -1;
          if (h.x.details && total > 0.f) {
            // process and element pick in the reference's order (src/MixedTransport.jl:131-140)
            float u = uni<float>(g) * total;
            const int last = nc - 1;
            int pick = last;
            for (int c = 0; c <= last; ++c) {
              u -= comp[c];
              if (u <= 0.f) {
                pick = c;
                break;
              }
            }
            h.x.pick = pick;
          }
        }
        __syncwarp();
      }
      if (live) {
        const int r = h.x.kind != CONT_NONE ? geo.template resume<PHASE>(h, g)
                                            : geo.template advance<true, PHASE>(h, g);
        live = settle(r, &i);
      }
      if (!__any_sync(0xffffffffu, live)) break;
    }
  } else {
    while (live) live = settle(geo.template advance<false, PHASE>(h, g), &i);
  }
}

// ------------------------------------------------------------ longest first
// The persistent loop hands histories out in counter order, and a warp runs
// until its last lane's history ends.  Handing the costly histories out
// first (a counting sort on a per-history cost bucket, descending) keeps the
// lanes of a warp on histories of similar length and leaves only short ones
// for the end of the launch.  A history's result does not depend on when or
// where it runs, so the order changes no result.
constexpr int kSchedBuckets = 1024;

// count[b] += number of items whose bucket is b (n items, or *n_dev when
// n_dev is set); bucket_of(s) gives the bucket of item s.  The lanes of a
// warp that share a bucket add once (many items often share one bucket).
template <class F>
__global__ void __launch_bounds__(256) sched_count_kernel(long n, const unsigned long long* n_dev,
                                                          F bucket_of, uint32_t* count) {
  __shared__ uint32_t h[kSchedBuckets];
  for (int b = threadIdx.x; b < kSchedBuckets; b += blockDim.x) h[b] = 0;
  __syncthreads();
  const long m = n_dev ? long(*n_dev) : n;
  const int lane = threadIdx.x & 31;
  // warp-uniform loop over 32-item groups
  for (long s0 = blockIdx.x * long(blockDim.x) + (threadIdx.x & ~31); s0 < m;
       s0 += long(gridDim.x) * blockDim.x) {
    const long s = s0 + lane;
    const int b = s < m ? bucket_of(s) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    if (b >= 0 && lane == __ffs(peers) - 1) atomicAdd(&h[b], uint32_t(__popc(peers)));
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kSchedBuckets; b += blockDim.x)
    if (h[b]) atomicAdd(&count[b], h[b]);
}
// offset[b] = items in buckets above b (descending exclusive scan); one block
// of kSchedBuckets threads.
static __global__ void __launch_bounds__(kSchedBuckets) sched_scan_kernel(const uint32_t* count,
                                                                   uint32_t* offset) {
  __shared__ uint32_t s[kSchedBuckets];
  const int t = threadIdx.x;
  s[t] = count[kSchedBuckets - 1 - t];  // descending bucket order
  __syncthreads();
  for (int d = 1; d < kSchedBuckets; d <<= 1) {
    const uint32_t v = t >= d ? s[t - d] : 0u;
    __syncthreads();
    s[t] += v;
    __syncthreads();
  }
  offset[kSchedBuckets - 1 - t] = s[t] - count[kSchedBuckets - 1 - t];
}
// order[offset[b]++] = s for every item s of bucket b (the lanes of a warp
// that share a bucket take consecutive places with one atomic).
template <class F>
__global__ void __launch_bounds__(256) sched_scatter_kernel(long n, const unsigned long long* n_dev,
                                                            F bucket_of, uint32_t* offset,
                                                            uint32_t* order) {
  const long m = n_dev ? long(*n_dev) : n;
  const int lane = threadIdx.x & 31;
  for (long s0 = blockIdx.x * long(blockDim.x) + (threadIdx.x & ~31); s0 < m;
       s0 += long(gridDim.x) * blockDim.x) {
    const long s = s0 + lane;
    const int b = s < m ? bucket_of(s) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, b);
    const int leader = __ffs(peers) - 1;
    uint32_t at = 0;
    if (b >= 0 && lane == leader) at = atomicAdd(&offset[b], uint32_t(__popc(peers)));
    at = __shfl_sync(0xffffffffu, at, leader);
    if (b >= 0) order[at + __popc(peers & ((1u << lane) - 1u))] = uint32_t(s);
  }
}
// Longest-first order of n items (or *n_dev items: the count of a queue
// filled on the device), count and offset 2 x kSchedBuckets words of
// scratch; three launches on the stream.
template <class F>
inline cudaError_t sched_order(cudaStream_t st, long n, const unsigned long long* n_dev,
                               F bucket_of, uint32_t* count, uint32_t* order, long long* launches) {
  cudaError_t e = cudaMemsetAsync(count, 0, kSchedBuckets * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  const int blocks = int(std::min<long>((n + 255) / 256, 152L * 4));
  sched_count_kernel<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(n, n_dev, bucket_of, count);
  sched_scan_kernel<<<1, kSchedBuckets, 0, st>>>(count, count + kSchedBuckets);
  sched_scatter_kernel<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(n, n_dev, bucket_of,
                                                               count + kSchedBuckets, order);
  *launches += 3;
  return cudaGetLastError();
}

}  // namespace mc
}  // namespace dp
