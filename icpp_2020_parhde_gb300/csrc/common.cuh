// common.cuh -- device helpers shared by the layout kernels (sm_103a).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "parhde.h"

#define PHDE_FULL_MASK 0xffffffffu

typedef unsigned long long ull;

// ---------------------------------------------------------------------------------------------
// Grid-wide barrier for cooperative launches.
//
// Monotonic arrival counter: thread 0 of every block adds 1 with release semantics (after bar.sync, so
// the whole block's writes are ordered before it), then polls the counter with acquire loads until it
// reaches the next multiple of the number of blocks; the closing bar.sync orders the block's threads
// after that acquire.  One round trip to arrive, one to observe -- no reset, no generation word.  The
// counter is zeroed before each launch (phde_reset_sync); 2^32 arrivals bound the barriers per launch.
//
// Every wait is bounded: after `timeout_ns` of %globaltimer the waiting thread records
// PHDE_ERR_TIMEOUT in the kernel's error word and the block returns false; a block that sees any error
// word also returns false.  Callers leave the kernel on false, so a kernel never spins forever.
struct GridSync {
  unsigned int count;
  unsigned int spare;
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned atom_add_release_u32(unsigned *p, unsigned v) {
  unsigned old;
  asm volatile("atom.release.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ int ld_volatile_i32(const int *p) { return *(const volatile int *)p; }
__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// `expected` is the number of blocks that must arrive (gridDim.x for a real barrier).
__device__ __forceinline__ bool grid_barrier(GridSync *gs, int *err, uint64_t timeout_ns, unsigned expected) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned arrived = atom_add_release_u32(&gs->count, 1u);
    const unsigned target = (arrived / expected + 1u) * expected;
    if (ld_acquire_u32(&gs->count) - target > 0x80000000u) {  // not yet reached (wrap-safe compare)
      const uint64_t t0 = global_timer_ns();
      unsigned spins = 0;
      while (ld_acquire_u32(&gs->count) - target > 0x80000000u) {
        if ((++spins & 7u) == 0) {
          if (ld_volatile_i32(err) != 0) {
            ok = 0;
            break;
          }
          if (global_timer_ns() - t0 > timeout_ns) {
            atomicCAS(err, 0, PHDE_ERR_TIMEOUT);
            ok = 0;
            break;
          }
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ bool grid_sync(GridSync *gs, int *err, uint64_t timeout_ns) {
  return grid_barrier(gs, err, timeout_ns, gridDim.x);
}

// ---------------------------------------------------------------------------------------------
// L2 eviction priorities.  A policy word from createpolicy rides on loads and reductions as a hint: data
// gathered again and again (a search frontier) is marked evict-last, data streamed once (adjacency lists,
// write-once records) evict-first, so the streams do not push the reused data out of L2.  Hints only: the
// values read and written are the same with or without them.
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
// 16 bytes through L2 only (never a possibly stale L1 line: other blocks write these words between grid
// barriers), with an L2 policy
__device__ __forceinline__ uint4 ld_cg_hint(const void *p, uint64_t pol) {
  uint4 v;
  asm volatile("ld.global.cg.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p), "l"(pol));
  return v;
}
// read-only 16 bytes with an L2 policy
__device__ __forceinline__ uint4 ld_nc_hint16(const void *p, uint64_t pol) {
  uint4 v;
  asm volatile("ld.global.nc.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p), "l"(pol));
  return v;
}
// read-only 4 bytes (the adjacency) with an L2 policy
__device__ __forceinline__ uint32_t ld_nc_hint(const uint32_t *p, uint64_t pol) {
  uint32_t v;
  asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}
// 32 bytes (four 64-bit words) in one 256-bit load through L2 only, with an L2 policy; p 32-byte aligned
__device__ __forceinline__ void ld_cg_hint32(const void *p, uint64_t pol, unsigned long long (&x)[4]) {
  asm volatile("ld.global.cg.L2::cache_hint.v4.u64 {%0, %1, %2, %3}, [%4], %5;"
               : "=l"(x[0]), "=l"(x[1]), "=l"(x[2]), "=l"(x[3])
               : "l"(p), "l"(pol));
}
// Asynchronous global -> shared copies (cp.async): 16 bytes through L2 only, or 8 bytes; a group per commit.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)), "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most `n` of this thread's committed groups are still in flight
template <int n>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(n) : "memory"); }

// OR-reduction in L2 (no value returned) with an L2 policy
__device__ __forceinline__ void red_or_hint(unsigned long long *p, unsigned long long v, uint64_t pol) {
  asm volatile("red.global.or.L2::cache_hint.b64 [%0], %1, %2;" ::"l"(p), "l"(v), "l"(pol) : "memory");
}

// ---------------------------------------------------------------------------------------------
// Reductions.
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(PHDE_FULL_MASK, v, o);
  return v;
}

__device__ __forceinline__ ull warp_max_u64(ull v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ull w = __shfl_xor_sync(PHDE_FULL_MASK, v, o);
    v = w > v ? w : v;
  }
  return v;
}

__device__ __forceinline__ unsigned warp_max_u32(unsigned v) { return __reduce_max_sync(PHDE_FULL_MASK, v); }

// Block sum of one value per thread; result valid in every thread.  `scratch` holds >= 32 entries.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T *scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  T r = 0;
  for (int w = 0; w < nw; w++) r += scratch[w];  // fixed order: deterministic
  return r;
}

__device__ __forceinline__ ull block_max_u64(ull v, ull *scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_max_u64(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  ull r = 0;
  for (int w = 0; w < nw; w++) r = scratch[w] > r ? scratch[w] : r;
  return r;
}

// ---------------------------------------------------------------------------------------------
// Block-aggregated append to a frontier queue.  Each flagged thread appends vertex v with out-degree
// dv.  One 64-bit atomic per block advances both the slot count (high 32 bits) and the running edge
// total (low 32 bits), so the start-edge array qe[] is non-decreasing in slot order -- that is what
// lets the next top-down step find the owner of an edge by binary search.  Edge totals stay below
// 2^32 because nnz < 2^32 (uint32 adjacency).  Must be called by every thread of the block.
struct PushScratch {
  ull warp_tot[32];
  ull base;
};

__device__ __forceinline__ void block_push(bool flag, uint32_t v, uint32_t dv, uint32_t *qv, uint32_t *qe, ull *ctr,
                                           PushScratch *sc) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const ull mine = flag ? ((1ull << 32) | (ull)dv) : 0ull;
  ull x = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    ull y = __shfl_up_sync(PHDE_FULL_MASK, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sc->warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    ull w = lane < nw ? sc->warp_tot[lane] : 0ull;
    ull incl = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      ull y = __shfl_up_sync(PHDE_FULL_MASK, incl, o);
      if (lane >= o) incl += y;
    }
    ull total = __shfl_sync(PHDE_FULL_MASK, incl, 31);
    if (lane < nw) sc->warp_tot[lane] = incl - w;  // exclusive prefix per warp
    if (lane == 0) sc->base = total ? atomicAdd(ctr, total) : 0ull;
  }
  __syncthreads();
  if (flag) {
    ull pos = sc->base + sc->warp_tot[warp] + (x - mine);
    uint32_t slot = (uint32_t)(pos >> 32);
    qv[slot] = v;
    qe[slot] = (uint32_t)(pos & 0xffffffffull);
  }
  __syncthreads();
}

// Largest index s in [0, f) with qe[s] <= e (qe non-decreasing, qe[0] == 0).
__device__ __forceinline__ uint32_t owner_slot(const uint32_t *qe, uint32_t f, uint32_t e) {
  uint32_t lo = 0, hi = f;  // invariant: qe[lo] <= e, answer in [lo, hi)
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (qe[mid] <= e)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Largest s in [0, f) with qe[s] <= e (qe non-decreasing, qe[0] == 0, every lane passes the same e): a
// 32-ary search by the whole warp, one probe per lane and step, about log32(f) dependent loads instead of
// the log2(f) of owner_slot.
//
// Owners of the 32 consecutive edges e0 + lane (lane = 0..31) of a warp, found by the whole warp (every
// lane calls it with the same e0 < total edges).  The warp's first owner comes from the 32-ary search;
// the others from one window
// load qe[s0 .. s0+31]: the slot starting at edge e0 + t is written to position t of a per-warp scratch
// (the largest such slot, for slots of zero out-degree), and a prefix maximum over the lanes gives each
// lane the last slot starting at or before its edge.  A lane whose edge lies beyond the window (only
// possible with zero-degree frontier entries) falls back to the binary search.  `win` is 32 words of
// shared memory private to the warp; `start` receives qe[owner].
__device__ __forceinline__ uint32_t warp_search_slot(const uint32_t *qe, uint32_t f, uint32_t e) {
  const int lane = threadIdx.x & 31;
  uint32_t lo = 0, hi = f;  // invariant: qe[lo] <= e, answer in [lo, hi)
  while (hi - lo > 32) {
    const uint32_t step = (hi - lo + 31) >> 5;
    const uint32_t pos = lo + (uint32_t)lane * step;
    const unsigned m = __ballot_sync(PHDE_FULL_MASK, pos < hi && qe[pos] <= e);  // bit 0 always set
    lo += (uint32_t)(31 - __clz(m)) * step;
    hi = min(hi, lo + step);
  }
  const uint32_t pos = lo + lane;
  const unsigned m = __ballot_sync(PHDE_FULL_MASK, pos < hi && qe[pos] <= e);
  return lo + (uint32_t)(31 - __clz(m));
}

__device__ __forceinline__ uint32_t warp_owner_slots(const uint32_t *qe, uint32_t f, uint32_t e0, uint32_t *win,
                                                     uint32_t &start) {
  const int lane = threadIdx.x & 31;
  const uint32_t lo = warp_search_slot(qe, f, e0);
  const uint32_t s0 = lo, sl = s0 + lane;
  const uint32_t q = sl < f ? qe[sl] : 0xffffffffu;
  const uint32_t qx = s0 + 32 < f ? qe[s0 + 32] : 0xffffffffu;
  win[lane] = 0;
  __syncwarp();
  if (q != 0xffffffffu && q >= e0 && q - e0 < 32u) atomicMax(win + (q - e0), (uint32_t)lane);
  __syncwarp();
  uint32_t off = win[lane];
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(PHDE_FULL_MASK, off, o);
    if (lane >= o) off = max(off, y);
  }
  __syncwarp();  // win is reused by the next call
  const uint32_t e = e0 + lane;
  start = __shfl_sync(PHDE_FULL_MASK, q, (int)off);  // qe of the owner, from the window
  if (e >= qx) {
    const uint32_t s = owner_slot(qe, f, e);
    start = qe[s];
    return s;
  }
  return s0 + off;
}

// block_push for two queues at once: the near frontier (vertex + start-edge prefix, as block_push, and
// optionally a third per-slot word o) and a plain vertex list (the far pile), one scan and one barrier pair
// for both, the two counter atomics issued by two lanes together.
struct Push2Scratch {
  ull warp_tot[32];
  unsigned warp_far[32];
  ull base;
  unsigned base_far;
};

__device__ __forceinline__ void block_push2(bool to_near, uint32_t v, uint32_t dv, uint32_t *qv, uint32_t *qe,
                                            ull *ctr, bool to_far, uint32_t *far, unsigned *far_ctr,
                                            Push2Scratch *sc, uint32_t *qo = nullptr, uint32_t o = 0) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const ull mine = to_near ? ((1ull << 32) | (ull)dv) : 0ull;
  ull x = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    ull y = __shfl_up_sync(PHDE_FULL_MASK, x, o);
    if (lane >= o) x += y;
  }
  const unsigned fb = __ballot_sync(PHDE_FULL_MASK, to_far);
  if (lane == 31) {
    sc->warp_tot[warp] = x;
    sc->warp_far[warp] = __popc(fb);
  }
  __syncthreads();
  if (warp == 0) {
    const ull w = lane < nw ? sc->warp_tot[lane] : 0ull;
    const unsigned wf = lane < nw ? sc->warp_far[lane] : 0u;
    ull incl = w;
    unsigned inclf = wf;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const ull y = __shfl_up_sync(PHDE_FULL_MASK, incl, o);
      const unsigned yf = __shfl_up_sync(PHDE_FULL_MASK, inclf, o);
      if (lane >= o) {
        incl += y;
        inclf += yf;
      }
    }
    const ull total = __shfl_sync(PHDE_FULL_MASK, incl, 31);
    const unsigned totf = __shfl_sync(PHDE_FULL_MASK, inclf, 31);
    if (lane < nw) {
      sc->warp_tot[lane] = incl - w;
      sc->warp_far[lane] = inclf - wf;
    }
    if (lane == 0) sc->base = total ? atomicAdd(ctr, total) : 0ull;
    if (lane == 1) sc->base_far = totf ? atomicAdd(far_ctr, totf) : 0u;
  }
  __syncthreads();
  if (to_near) {
    const ull pos = sc->base + sc->warp_tot[warp] + (x - mine);
    const uint32_t slot = (uint32_t)(pos >> 32);
    qv[slot] = v;
    qe[slot] = (uint32_t)(pos & 0xffffffffull);
    if (qo) qo[slot] = o;
  }
  if (to_far) far[sc->base_far + sc->warp_far[warp] + __popc(fb & ((1u << lane) - 1u))] = v;
  __syncthreads();
}

// ---------------------------------------------------------------------------------------------
// Host-side helpers.
struct LaunchCounter {
  long long n = 0;
};
