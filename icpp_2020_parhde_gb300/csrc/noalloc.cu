// noalloc.cu -- a breadth-first search that performs no device memory allocation.
//
// Who this is for: callers that are not allowed to call cudaMalloc.  Typical cases are a host
// application whose own memory pool owns all device memory (a private cudaMalloc would compete with the
// pool or break its accounting), code on a latency-critical path where cudaMalloc/cudaFree would
// synchronise the device, and plugins that are only ever handed pre-allocated device buffers.
//
// phde_bfs_noalloc takes the CSR graph and the output distance column as device pointers plus a CUDA
// stream.  Everything else the kernel needs -- two frontier queues with their edge-prefix arrays, the
// frontier counters, the grid barrier and the error word -- lives in ONE file-scope __device__ array,
// g_noalloc_scratch, sized for PHDE_NOALLOC_MAX_VERTICES vertices (16 MiB + 256 bytes).  Every GPU
// that loads this library holds that array until the process exits.  All calls share it and it keeps
// the previous call's contents, so each call clears the parts that must start at zero; two calls
// whose kernels overlap on the GPU (for example on two streams) race on the shared array and must
// be serialised by the caller.
//
// Host code cannot use the array's name as a device address (the name denotes a host-side stand-in);
// on the first call on each device, with that device current, the entry point asks the runtime for
// the array's device address with cudaGetSymbolAddress and caches it.  That first call therefore does
// one-time set-up and should come before any stream capture.
#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "parhde.h"

namespace {

constexpr int NA_THREADS = 512;
constexpr int64_t NA_MAX_N = PHDE_NOALLOC_MAX_VERTICES;
constexpr size_t NA_QUEUE_BYTES = sizeof(uint32_t) * (size_t)NA_MAX_N;
constexpr size_t NA_CTRL_OFFSET = 4 * NA_QUEUE_BYTES;  // after qv0, qv1, qe0, qe1
constexpr size_t NA_CTRL_BYTES = 256;                  // ctr[4] (32 B), GridSync (8 B), err (4 B), padding
constexpr size_t NA_SCRATCH_BYTES = NA_CTRL_OFFSET + NA_CTRL_BYTES;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_SCRATCH_BYTES];

struct NaArgs {
  const int64_t *off;
  const uint32_t *adj;
  int64_t n, nnz, src;
  int32_t *dist;  // caller's column, filled with -1 before the launch
  uint32_t *qv0, *qv1, *qe0, *qe1;
  ull *ctr;
  GridSync *gs;
  int *err;
  uint64_t timeout_ns;
};

// Direction-optimising BFS from one source (the rule of gapbs/bfs.cc:159-183, alpha 15, beta 18),
// one persistent cooperative launch, bounded grid barriers between levels.
__global__ void __launch_bounds__(NA_THREADS) bfs_noalloc_kernel(NaArgs a) {
  __shared__ PushScratch psc;
  const int64_t n = a.n;
  const int tid = threadIdx.x;
  const int64_t gstride = (int64_t)gridDim.x * blockDim.x, gbase = (int64_t)blockIdx.x * blockDim.x;
  if (tid == 0) a.dist[a.src] = 0;
  __syncthreads();
  const int64_t s_off = a.off[a.src];
  uint32_t f_cnt = 1, f_edges = (uint32_t)(a.off[a.src + 1] - s_off);
  int64_t edges_to_check = a.nnz, scout = f_edges, awake = 0, old_awake = 0;
  bool in_bu = false;
  for (int32_t L = 0; f_cnt > 0; L++) {
    if (!in_bu) {
      if (scout > edges_to_check / 15) {
        in_bu = true;
        awake = f_cnt;
      } else {
        edges_to_check -= scout;
      }
    }
    if (in_bu) old_awake = awake;
    const uint32_t *qin_v = (L & 1) ? a.qv1 : a.qv0, *qin_e = (L & 1) ? a.qe1 : a.qe0;
    uint32_t *qout_v = (L & 1) ? a.qv0 : a.qv1, *qout_e = (L & 1) ? a.qe0 : a.qe1;
    ull *octr = a.ctr + (L & 3);
    if (blockIdx.x == 0 && tid == 0) a.ctr[(L + 2) & 3] = 0ull;
    if (!in_bu) {
      const int64_t E = f_edges;
      for (int64_t base = gbase; base < E; base += gstride) {
        const int64_t e = base + tid;
        bool claimed = false;
        uint32_t v = 0, dv = 0;
        if (e < E) {
          int64_t j;
          if (L == 0) {
            j = s_off + e;
          } else {
            const uint32_t s = owner_slot(qin_e, f_cnt, (uint32_t)e);
            j = a.off[qin_v[s]] + (e - (int64_t)qin_e[s]);
          }
          v = __ldg(a.adj + j);
          if (a.dist[v] == -1 && atomicCAS(a.dist + v, -1, L + 1) == -1) {
            claimed = true;
            dv = (uint32_t)(a.off[v + 1] - a.off[v]);
          }
        }
        block_push(claimed, v, dv, qout_v, qout_e, octr, &psc);
      }
    } else {
      for (int64_t base = gbase; base < n; base += gstride) {
        const int64_t v = base + tid;
        bool found = false;
        uint32_t dv = 0;
        if (v < n && a.dist[v] == -1) {
          const int64_t j0 = a.off[v], j1 = a.off[v + 1];
          for (int64_t j = j0; j < j1; j++)
            if (a.dist[__ldg(a.adj + j)] == L) {
              found = true;
              break;
            }
          if (found) {
            a.dist[v] = L + 1;
            dv = (uint32_t)(j1 - j0);
          }
        }
        block_push(found, (uint32_t)v, dv, qout_v, qout_e, octr, &psc);
      }
    }
    if (!grid_sync(a.gs, a.err, a.timeout_ns)) return;
    const ull out = __ldcg(octr);
    f_cnt = (uint32_t)(out >> 32);
    f_edges = (uint32_t)(out & 0xffffffffull);
    if (in_bu) {
      awake = f_cnt;
      if (!(awake >= old_awake || awake > n / 18)) {
        in_bu = false;
        scout = 1;
      }
    } else {
      scout = f_edges;
    }
  }
}

// Device address of g_noalloc_scratch, looked up once per device.
std::mutex g_na_mutex;
unsigned char *g_na_addr[64] = {};

int scratch_address(int dev, unsigned char **out) {
  if (dev < 0 || dev >= 64) return PHDE_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return PHDE_ERR_CUDA;
    }
    g_na_addr[dev] = (unsigned char *)p;
  }
  *out = g_na_addr[dev];
  return PHDE_OK;
}

}  // namespace

extern "C" int phde_bfs_noalloc(const int64_t *d_offsets, const uint32_t *d_adj, int64_t n, int64_t nnz,
                                int64_t source, int32_t *d_dist, void *stream) {
  if (!d_offsets || !d_adj || !d_dist || n < 1 || nnz < 0 || source < 0 || source >= n) return PHDE_ERR_INVALID;
  if (n > NA_MAX_N || nnz >= (int64_t)0xffffffffll) {
    fprintf(stderr,
            "phde_bfs_noalloc: graph with n=%lld, nnz=%lld exceeds the fixed scratch capacity "
            "(at most %lld vertices and fewer than 2^32 adjacency entries)\n",
            (long long)n, (long long)nnz, (long long)NA_MAX_N);
    return PHDE_ERR_TOO_LARGE;
  }
  int dev = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return PHDE_ERR_CUDA;
  }
  unsigned char *base = nullptr;
  int rc = scratch_address(dev, &base);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char *ctrl = base + NA_CTRL_OFFSET;
  NaArgs a;
  a.off = d_offsets;
  a.adj = d_adj;
  a.n = n;
  a.nnz = nnz;
  a.src = source;
  a.dist = d_dist;
  a.qv0 = (uint32_t *)base;
  a.qv1 = (uint32_t *)(base + NA_QUEUE_BYTES);
  a.qe0 = (uint32_t *)(base + 2 * NA_QUEUE_BYTES);
  a.qe1 = (uint32_t *)(base + 3 * NA_QUEUE_BYTES);
  a.ctr = (ull *)ctrl;
  a.gs = (GridSync *)(ctrl + 32);
  a.err = (int *)(ctrl + 40);
  a.timeout_ns = 5000000000ull;
  if (cudaMemsetAsync(d_dist, 0xff, sizeof(int32_t) * (size_t)n, s) != cudaSuccess ||
      cudaMemsetAsync(ctrl, 0, NA_CTRL_BYTES, s) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bfs_noalloc_kernel, NA_THREADS, 0) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    return PHDE_ERR_CUDA;
  }
  per_sm = per_sm < 4 ? per_sm : 4;
  void *args[] = {&a};
  if (cudaLaunchCooperativeKernel((const void *)bfs_noalloc_kernel, dim3(nsm * per_sm), dim3(NA_THREADS), args, 0, s) !=
      cudaSuccess) {
    cudaGetLastError();
    return PHDE_ERR_CUDA;
  }
  int h_err = 0;
  if (cudaMemcpyAsync(&h_err, a.err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return PHDE_ERR_CUDA;
  }
  return h_err;  // PHDE_OK, or PHDE_ERR_TIMEOUT if a bounded barrier wait gave up
}
