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
//   int advance<COOP, PHASE>(Hist&, Stream&)  one step: ADV_*
//   int resume<PHASE>(Hist&, Stream&)         finish a suspended step: ADV_*
#pragma once
#include <cooperative_groups.h>

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

// First of the next `batch` history indices for the calling thread
// (warp-aggregated atomic: the active threads take consecutive runs).
__device__ __forceinline__ long next_history(unsigned long long* counter, int batch = 1) {
  namespace cg = cooperative_groups;
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned long long base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, (unsigned long long)g.size() * batch);
  base = g.shfl(base, 0);
  return long(base + (unsigned long long)g.thread_rank() * batch);
}

// A block whose table staging gave up takes its share of the phase's
// histories all the same and ends each one flagged DP_ST_TABLE_WAIT (no flux,
// no table read), so that every history of the launch is accounted for.
template <class R, int PHASE, class G>
__device__ __forceinline__ void drain_histories(G& geo, const Consts& C,
                                                unsigned long long* counter,
                                                typename G::Queue* queue) {
  const long n = PHASE == 0 ? geo.n0() : long(*(volatile unsigned long long*)(counter + 2));
  typename G::Hist h;
  Stream g;
  for (;;) {
    const long j0 = next_history(counter + PHASE, C.batch);
    if (j0 >= n) break;
    for (long j = j0; j < j0 + C.batch && j < n; ++j) {
      long i = j;
      if (PHASE == 0) geo.start(j, h, g);
      else i = geo.load(queue[j], h, g);
      h.s.status |= ST_TABLE;
      geo.end(i, h);
    }
  }
}

// Runs histories until none is left for this phase.  counter[PHASE] hands out
// history indices, counter[2] counts the hand-off queue.  With COOP, `item`
// and `comp` are this warp's DCS buffers in shared memory.
template <class R, int PHASE, bool COOP, class G>
__device__ __forceinline__ void transport_histories(G& geo, const Consts& C,
                                                    unsigned long long* counter,
                                                    typename G::Queue* queue, float* item,
                                                    float* comp) {
  const long n = PHASE == 0 ? geo.n0() : long(*(volatile unsigned long long*)(counter + 2));
  typename G::Hist h;
  Stream g;
  // a thread takes C.batch (1, 2 or 4) consecutive histories from the
  // counter at a time; the counter only moves in multiples of it, so a run
  // starts at a multiple of C.batch (a history's result does not depend on
  // the thread that runs it)
  long cur = -1;
  auto take = [&](long* idx) -> bool {
    long j;
    if (cur >= 0 && ((cur + 1) & (C.batch - 1)) != 0) j = ++cur;
    else j = cur = next_history(counter + PHASE, C.batch);
    if (j >= n) return false;
    if (PHASE == 0) {
      *idx = j;
      geo.start(j, h, g);
    } else {
      *idx = geo.load(queue[j], h, g);
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
    const int lane = threadIdx.x & 31;
    for (;;) {
      // serve the hard events the warp's suspended steps wait for, one at a time
      unsigned want = __ballot_sync(0xffffffffu, live && h.x.kind != CONT_NONE);
      while (want) {
        const int L = __ffs(want) - 1;
        want &= want - 1;
        const int med = __shfl_sync(0xffffffffu, h.x.medium, L);
        const double anc = __shfl_sync(0xffffffffu, h.x.anc, L);
        const double q = __shfl_sync(0xffffffffu, h.x.q, L);
        const Med<R>& m = geo.medium(med);
        const double total = coop_total(m.elf, m.nel, float(C.mass), anc, q, item, comp);
        if (lane == L) {
          h.x.total = total;
          h.x.pick = -1;
          if (h.x.details && total > 0.0) {
            // process and element pick in the reference's order (src/MixedTransport.jl:131-140)
            double u = uni_d(g) * total;
            const int last = 4 * m.nel - 1;
            int pick = last;
            for (int c = 0; c <= last; ++c) {
              u -= double(comp[c]);
              if (u <= 0.0) {
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

}  // namespace mc
}  // namespace dp
