// eigen.cu -- the k x k symmetric eigensolve, one CTA, FP64.
//
// power_kernel: the reference's non-MKL eigensolver (ParallelComponents.cpp:48-158, reached through
//   compute_eigens, DrawingBase.cpp:39-108): N start vectors rand()/RAND_MAX after srand(1), repeated
//   multiply-by-K, Gram-Schmidt of every vector against the ones before it, renormalisation, stop when
//   every vector moved less than |cos| = 0.999; output columns in ascending |eigenvalue| order with the
//   reference's sign rule.  The glibc rand() stream is regenerated on the device (the published TYPE_3
//   additive-feedback generator).  The multiply keeps the reference's summation order; the Gram-Schmidt
//   runs as a wavefront (vector i takes its projection onto vector j at step i+j, when vector j is final),
//   so its N(N-1)/2 dependent projections take 2N-3 block-synchronous steps.
// jacobi_kernel: exact solve (the LAPACKE_dsyev role of the MKL build): cyclic Jacobi on the symmetric
//   part with the round-robin pairing, N/2 disjoint rotations per step; eigenvalues ascending; every
//   eigenvector signed so that its largest-magnitude entry (lowest index on ties) is positive.
// pick_kernel: eigenVectors columns for First (0..c-1) or Largest (N-1-j), DrawingBase.cpp:51-108.
#include <algorithm>
#include <cooperative_groups.h>
#include <cstdio>
#include <cstdlib>

#include "ctx.h"

namespace {

constexpr int EIG_THREADS = 1024;

// <a, b> for one warp.  SEQ: lane 0 sums in index order with separate roundings (the reference's
// one-thread prodSeq / normL2, ParallelComponents.cpp:13-46) and broadcasts; otherwise a lane-strided
// sum and a shuffle tree.
template <bool SEQ>
__device__ __forceinline__ double warp_dot(const double *a, const double *b, int N, int lane) {
  if (SEQ) {
    double s = 0;
    if (lane == 0)
      for (int r = 0; r < N; r++) s = __dadd_rn(s, __dmul_rn(a[r], b[r]));
    return __shfl_sync(PHDE_FULL_MASK, s, 0);
  }
  double s = 0;
  for (int r = lane; r < N; r += 32) s = fma(a[r], b[r], s);
  return warp_sum(s);
}

// Work arrays live in global memory (a few N*N doubles, L2/L1 resident); dd caches <E_j, E_j>.
template <bool SEQ>
__global__ void __launch_bounds__(EIG_THREADS) power_kernel(const double *Kin, int N, double *K, double *E,
                                                            double *T, double *evals, int *iters, int *status,
                                                            int max_iter, double *dd) {
  __shared__ double red[32];
  __shared__ double s_r;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int NN = N * N;
  for (int i = tid; i < NN; i += blockDim.x) K[i] = Kin[i];
  // start vectors: glibc rand() after srand(1), E[j + i*N] = r[i*N + j] / RAND_MAX (column i filled first)
  if (tid == 0) {
    int32_t ring[34];
    ring[0] = 1;
    for (int i = 1; i < 31; i++) {
      int32_t hi = ring[i - 1] / 127773, lo = ring[i - 1] % 127773;
      int32_t word = 16807 * lo - 2836 * hi;
      if (word < 0) word += 2147483647;
      ring[i] = word;
    }
    for (int i = 31; i < 34; i++) ring[i] = ring[i - 31];
    // r[i] for i >= 34 is r[i-31] + r[i-3]; keep the last 34 values in a ring indexed mod 34
    int out = 0;
    for (int i = 34; out < NN; i++) {
      const int32_t v = (int32_t)((uint32_t)ring[(i - 31) % 34] + (uint32_t)ring[(i - 3) % 34]);
      ring[i % 34] = v;
      if (i >= 344) {
        E[out] = (double)(int32_t)(((uint32_t)v) >> 1) / 2147483647.0;
        out++;
      }
    }
  }
  __syncthreads();
  for (int i = warp; i < N; i += nw) {
    const double nv = sqrt(warp_dot<SEQ>(E + i * N, E + i * N, N, lane));
    for (int r = lane; r < N; r += 32) E[r + i * N] = E[r + i * N] / nv;
    if (lane == 0) evals[i] = nv;
  }
  __syncthreads();
  double r = 0;
  int it = 0;
  while (r < 1.0 - 1e-3) {
    it++;
    if (isnan(r) || isinf(r) || it > max_iter) {
      if (tid == 0) *status = PHDE_ERR_NOCONVERGE;
      return;
    }
    for (int i = tid; i < NN; i += blockDim.x) T[i] = E[i];
    __syncthreads();
    // E[:, i] = K * T[:, i], accumulated over j in order (ParallelComponents.cpp:82-90)
    for (int idx = tid; idx < NN; idx += blockDim.x) {
      const int row = idx % N, col = idx / N;
      double s = 0;
      for (int j = 0; j < N; j++) s = __dadd_rn(s, __dmul_rn(K[row + j * N], T[j + col * N]));
      E[idx] = s;
    }
    __syncthreads();
    // Gram-Schmidt wavefront: at step t vector i projects out vector j = t - i (j < i).  Vector j is
    // final once t > 2j - 1; its <E_j, E_j> is cached the step it becomes final (t == 2j, i.e. when
    // vector i = j has no projection left to take).
    if (warp == 0) {
      const double d0 = warp_dot<SEQ>(E, E, N, lane);
      if (lane == 0) dd[0] = d0;
    }
    __syncthreads();
    for (int t = 1; t <= 2 * N - 2; t++) {
      for (int i = warp; i < N; i += nw) {
        const int j = t - i;
        if (j == i) {  // vector i just became final
          const double d = warp_dot<SEQ>(E + i * N, E + i * N, N, lane);
          if (lane == 0) dd[i] = d;
          continue;
        }
        if (j < 0 || j > i) continue;
        const double num = warp_dot<SEQ>(E + j * N, E + i * N, N, lane);
        const double fac = num / dd[j];
        for (int q = lane; q < N; q += 32) E[q + i * N] = __dsub_rn(E[q + i * N], __dmul_rn(fac, E[q + j * N]));
        __syncwarp();
      }
      __syncthreads();
    }
    for (int i = warp; i < N; i += nw) {
      const double nv = sqrt(warp_dot<SEQ>(E + i * N, E + i * N, N, lane));
      for (int q = lane; q < N; q += 32) E[q + i * N] = E[q + i * N] / nv;
      if (lane == 0) evals[i] = nv;
    }
    __syncthreads();
    // r = min_i |<E_i, T_i>|
    double mn = 1.0;
    for (int i = warp; i < N; i += nw) {
      double d = fabs(warp_dot<SEQ>(E + i * N, T + i * N, N, lane));
      mn = d < mn ? d : mn;
    }
    if (lane == 0) red[warp] = mn;
    __syncthreads();
    if (tid == 0) {
      double m = 1.0;
      for (int w = 0; w < nw; w++) m = red[w] < m ? red[w] : m;
      s_r = m;
    }
    __syncthreads();
    r = s_r;
  }
  __syncthreads();
  if (tid == 0) {  // ascending order of the norms (ParallelComponents.cpp:131-139)
    for (int a = 0, b = N - 1; a < b; a++, b--) {
      double t = evals[a];
      evals[a] = evals[b];
      evals[b] = t;
    }
    *iters = it;
    *status = PHDE_OK;
  }
  // K[:, N-1-i] = +-E[:, i]; the sign follows the first entry of E column N-1-i (ParallelComponents.cpp:140-153)
  for (int idx = tid; idx < NN; idx += blockDim.x) {
    const int i = idx / N, row = idx % N;
    const bool neg = E[(N - i - 1) * N] < 0;
    K[row + (N - i - 1) * N] = neg ? -E[row + i * N] : E[row + i * N];
  }
}

// ---- the same power iteration on a cluster of PW_CL CTAs (one per SM) ----
// GB300 runs FP64 at 1/64 of FP32, so one SM's FP64 pipe bounds the single-CTA kernel.  Here CTA c of
// the cluster owns vectors i = c, c + PW_CL, ...; each CTA keeps K in its shared memory, multiplies its
// own vectors, and in the Gram-Schmidt wavefront reads the finished vector j (and its cached <E_j,E_j>)
// straight from the owner's shared memory through distributed shared memory.  A hardware cluster
// barrier separates wavefront steps.  Every floating-point operation is the one power_kernel<false>
// performs, in the same order, so the two kernels return identical bits.
constexpr int PW_CL = 8;
constexpr int PW_MAX_N = 128;

__global__ void __cluster_dims__(PW_CL, 1, 1) __launch_bounds__(EIG_THREADS)
    power_cluster_kernel(const double *Kin, int N, double *Kout, double *evals_out, int *iters, int *status,
                         int max_iter) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  extern __shared__ double psm[];
  const int NO = (N + PW_CL - 1) / PW_CL;  // vectors owned per CTA
  double *Ks = psm;                         // N*N, column-major
  double *Eo = Ks + N * N;                  // NO*N: owned vector li at Eo + li*N
  double *To = Eo + NO * N;
  double *ddo = To + NO * N;                // NO
  double *evo = ddo + NO;                   // NO
  double *rmin = evo + NO;                  // 1 slot read by the whole cluster
  __shared__ double red[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int NN = N * N;
  for (int i = tid; i < NN; i += blockDim.x) Ks[i] = Kin[i];
  // start vectors: every CTA replays the glibc stream and keeps the columns it owns
  if (tid == 0) {
    int32_t ring[34];
    ring[0] = 1;
    for (int i = 1; i < 31; i++) {
      int32_t hi = ring[i - 1] / 127773, lo = ring[i - 1] % 127773;
      int32_t word = 16807 * lo - 2836 * hi;
      if (word < 0) word += 2147483647;
      ring[i] = word;
    }
    for (int i = 31; i < 34; i++) ring[i] = ring[i - 31];
    int out = 0;
    for (int i = 34; out < NN; i++) {
      const int32_t v = (int32_t)((uint32_t)ring[(i - 31) % 34] + (uint32_t)ring[(i - 3) % 34]);
      ring[i % 34] = v;
      if (i >= 344) {
        const int col = out / N, row = out % N;
        if (col % PW_CL == rank) Eo[(col / PW_CL) * N + row] = (double)(int32_t)(((uint32_t)v) >> 1) / 2147483647.0;
        out++;
      }
    }
  }
  __syncthreads();
  for (int li = warp; li < NO; li += nw) {
    const int i = rank + li * PW_CL;
    if (i >= N) continue;
    const double nv = sqrt(warp_dot<false>(Eo + li * N, Eo + li * N, N, lane));
    for (int r = lane; r < N; r += 32) Eo[li * N + r] = Eo[li * N + r] / nv;
    if (lane == 0) evo[li] = nv;
  }
  double r = 0;
  int it = 0;
  while (r < 1.0 - 1e-3) {
    it++;
    if (isnan(r) || isinf(r) || it > max_iter) {
      if (rank == 0 && tid == 0) *status = PHDE_ERR_NOCONVERGE;
      return;  // uniform across the cluster: every CTA holds the same r and it
    }
    __syncthreads();
    for (int x = tid; x < NO * N; x += blockDim.x) To[x] = Eo[x];
    __syncthreads();
    for (int idx = tid; idx < NO * N; idx += blockDim.x) {
      const int li = idx / N, row = idx % N;
      if (rank + li * PW_CL >= N) continue;
      double acc = 0;
      for (int j = 0; j < N; j++) acc = __dadd_rn(acc, __dmul_rn(Ks[row + j * N], To[j + li * N]));
      Eo[idx] = acc;
    }
    cluster.sync();
    if (rank == 0 && warp == 0) {  // vector 0 is final from the start
      const double d0 = warp_dot<false>(Eo, Eo, N, lane);
      if (lane == 0) ddo[0] = d0;
    }
    cluster.sync();
    for (int t = 1; t <= 2 * N - 2; t++) {
      for (int li = warp; li < NO; li += nw) {
        const int i = rank + li * PW_CL;
        const int j = t - i;
        if (i >= N || j < 0 || j > i) continue;
        if (j == i) {
          const double d = warp_dot<false>(Eo + li * N, Eo + li * N, N, lane);
          if (lane == 0) ddo[li] = d;
          continue;
        }
        const double *Ej = cluster.map_shared_rank(Eo, j % PW_CL) + (j / PW_CL) * N;
        const double djj = *cluster.map_shared_rank(ddo + j / PW_CL, j % PW_CL);
        const double num = warp_dot<false>(Ej, Eo + li * N, N, lane);
        const double fac = num / djj;
        for (int q = lane; q < N; q += 32) Eo[li * N + q] = __dsub_rn(Eo[li * N + q], __dmul_rn(fac, Ej[q]));
        __syncwarp();
      }
      cluster.sync();
    }
    double mn = 1.0;
    for (int li = warp; li < NO; li += nw) {
      const int i = rank + li * PW_CL;
      if (i >= N) continue;
      const double nv = sqrt(warp_dot<false>(Eo + li * N, Eo + li * N, N, lane));
      for (int q = lane; q < N; q += 32) Eo[li * N + q] = Eo[li * N + q] / nv;
      if (lane == 0) evo[li] = nv;
      __syncwarp();
      const double d = fabs(warp_dot<false>(Eo + li * N, To + li * N, N, lane));
      mn = d < mn ? d : mn;
    }
    if (lane == 0) red[warp] = mn;
    __syncthreads();
    if (tid == 0) {
      double m = 1.0;
      for (int w = 0; w < nw; w++) m = red[w] < m ? red[w] : m;
      *rmin = m;
    }
    cluster.sync();
    double m = 1.0;
    for (int c = 0; c < PW_CL; c++) {
      const double v = *cluster.map_shared_rank(rmin, c);
      m = v < m ? v : m;
    }
    r = m;
    cluster.sync();  // every CTA has read the slots before the next sweep overwrites them
  }
  // output: column N-1-i <- +-E_i, sign from the first entry of E_{N-1-i} (ParallelComponents.cpp:140-153);
  // eigenvalue norms reversed into ascending order
  for (int idx = tid; idx < NO * N; idx += blockDim.x) {
    const int li = idx / N, row = idx % N;
    const int i = rank + li * PW_CL;
    if (i >= N) continue;
    const int o = N - 1 - i;
    const double first = *cluster.map_shared_rank(Eo + (o / PW_CL) * N, o % PW_CL);
    Kout[row + o * N] = first < 0 ? -Eo[li * N + row] : Eo[li * N + row];
    if (row == 0) evals_out[o] = evo[li];
  }
  if (rank == 0 && tid == 0) {
    *iters = it;
    *status = PHDE_OK;
  }
  cluster.sync();  // keep every CTA's shared memory alive until the others have read it
}

// Exact symmetric eigensolve by parallel cyclic Jacobi (Brent-Luk round-robin ordering).
__global__ void __launch_bounds__(EIG_THREADS) jacobi_kernel(const double *Kin, int N, double *A, double *V,
                                                             double *K, double *evals, int *sweeps, int *status,
                                                             int max_sweeps) {
  __shared__ double red[32];
  __shared__ double s_cs[PHDE_MAX_K / 2 + 1], s_sn[PHDE_MAX_K / 2 + 1];
  __shared__ int s_p[PHDE_MAX_K / 2 + 1], s_q[PHDE_MAX_K / 2 + 1];
  __shared__ int s_order[PHDE_MAX_K + 1];
  __shared__ int s_done;
  __shared__ double s_off, s_tot;
  const int tid = threadIdx.x;
  const int M = (N + 1) & ~1;  // even number of slots; slot N (if any) is a dummy
  for (int idx = tid; idx < N * N; idx += blockDim.x) {
    const int i = idx % N, j = idx / N;
    A[idx] = 0.5 * (Kin[i + j * N] + Kin[j + i * N]);
    V[idx] = i == j ? 1.0 : 0.0;
  }
  for (int i = tid; i < M; i += blockDim.x) s_order[i] = i;
  __syncthreads();
  int sweep = 0;
  for (; sweep < max_sweeps; sweep++) {
    double off = 0, tot = 0;
    for (int idx = tid; idx < N * N; idx += blockDim.x) {
      const int i = idx % N, j = idx / N;
      const double a2 = A[idx] * A[idx];
      tot += a2;
      if (i != j) off += a2;
    }
    off = block_sum(off, red);
    tot = block_sum(tot, red);
    // converged when the off-diagonal Frobenius norm is below 1e-14 of the whole (squared: 1e-28)
    if (tid == 0) {
      s_done = (off <= 1e-28 * tot) || off == 0.0;
      s_off = off;
      s_tot = tot;
    }
    __syncthreads();
    if (s_done) break;
    for (int round = 0; round < M - 1; round++) {
      // circle method: slot m meets slot M-1-m; every pair meets once in M-1 rounds
      for (int m = tid; m < M / 2; m += blockDim.x) {
        int p = s_order[m], q = s_order[M - 1 - m];
        if (p > q) {
          int t = p;
          p = q;
          q = t;
        }
        double cs = 1.0, sn = 0.0;
        if (q < N) {
          const double apq = A[p + q * N];
          if (apq != 0.0) {
            const double app = A[p + p * N], aqq = A[q + q * N];
            const double theta = (aqq - app) / (2.0 * apq);
            const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
            cs = 1.0 / sqrt(t * t + 1.0);
            sn = t * cs;
          }
        }
        s_p[m] = p;
        s_q[m] = q;
        s_cs[m] = cs;
        s_sn[m] = sn;
      }
      __syncthreads();
      // A <- A J (columns p, q) and V <- V J
      for (int idx = tid; idx < (M / 2) * N; idx += blockDim.x) {
        const int m = idx / N, row = idx % N;
        const int p = s_p[m], q = s_q[m];
        if (q >= N || s_sn[m] == 0.0) continue;
        const double cs = s_cs[m], sn = s_sn[m];
        const double akp = A[row + p * N], akq = A[row + q * N];
        A[row + p * N] = cs * akp - sn * akq;
        A[row + q * N] = sn * akp + cs * akq;
        const double vkp = V[row + p * N], vkq = V[row + q * N];
        V[row + p * N] = cs * vkp - sn * vkq;
        V[row + q * N] = sn * vkp + cs * vkq;
      }
      __syncthreads();
      // A <- J^T A (rows p, q)
      for (int idx = tid; idx < (M / 2) * N; idx += blockDim.x) {
        const int m = idx / N, col = idx % N;
        const int p = s_p[m], q = s_q[m];
        if (q >= N || s_sn[m] == 0.0) continue;
        const double cs = s_cs[m], sn = s_sn[m];
        const double apk = A[p + col * N], aqk = A[q + col * N];
        A[p + col * N] = cs * apk - sn * aqk;
        A[q + col * N] = sn * apk + cs * aqk;
      }
      __syncthreads();
      // round-robin rotation of the slots, slot 0 fixed
      if (tid == 0) {
        const int last = s_order[M - 1];
        for (int i = M - 1; i > 1; i--) s_order[i] = s_order[i - 1];
        s_order[1] = last;
      }
      __syncthreads();
    }
  }
  if (tid == 0) {
    // ascending selection sort of the diagonal (stable on ties)
    for (int i = 0; i < N; i++) s_order[i] = i;
    for (int i = 0; i < N; i++) {
      int b = i;
      for (int j = i + 1; j < N; j++)
        if (A[s_order[j] + s_order[j] * N] < A[s_order[b] + s_order[b] * N]) b = j;
      const int t = s_order[i];
      s_order[i] = s_order[b];
      s_order[b] = t;
    }
    for (int c = 0; c < N; c++) evals[c] = A[s_order[c] + s_order[c] * N];
    *sweeps = sweep;
    // after the sweep cap, accept an off-diagonal norm below 1e-10 of the whole (squared: 1e-20)
    *status = (sweep < max_sweeps || s_off <= 1e-20 * s_tot) ? PHDE_OK : PHDE_ERR_NOCONVERGE;
  }
  __syncthreads();
  const int lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int c = warp; c < N; c += nw) {
    const int src = s_order[c];
    // index of the largest |entry| (lowest index on ties)
    double best = -1.0;
    int arg = 0;
    for (int i = lane; i < N; i += 32) {
      const double a = fabs(V[i + src * N]);
      if (a > best) {
        best = a;
        arg = i;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double b2 = __shfl_xor_sync(PHDE_FULL_MASK, best, o);
      const int a2 = __shfl_xor_sync(PHDE_FULL_MASK, arg, o);
      if (b2 > best || (b2 == best && a2 < arg)) {
        best = b2;
        arg = a2;
      }
    }
    const double sg = V[arg + src * N] < 0 ? -1.0 : 1.0;
    for (int i = lane; i < N; i += 32) K[i + c * N] = sg * V[i + src * N];
  }
}

// ---- shared-memory Jacobi for N <= JS_MAX_N: FP32 sweeps, FP64 re-orthonormalisation, FP64 sweeps ----
//
// GB300 issues FP64 at 1/64 of its FP32 rate, and a cyclic Jacobi solve of a k x k matrix is about ten
// sweeps of N-1 rounds.  Here the sweeps that only shrink the off-diagonal run in FP32 (A32, V32); the FP32
// eigenbasis V is then made orthonormal in FP64 (classical Gram-Schmidt, exact enough for a basis that is
// orthogonal to FP32 rounding), A is replaced by the exactly similar V^T A V computed in FP64, and FP64
// sweeps (quadratically convergent from an off-diagonal of FP32 rounding size) finish with the same
// convergence test as the global-memory kernel.  Everything lives in shared memory.
constexpr int JS_MIN_THREADS = 256;  // the shared-memory solver runs with 256..1024 threads
constexpr int JS_MAX_N = 96;  // 24 N (N|1) bytes of shared memory: A64, V64 and one work matrix
constexpr int JS_BAD_CAP = 512;       // unseparated pairs the targeted FP64 rotations take on (more: sweeps)
constexpr int JS_TJ_MAX_ROUNDS = 48;  // rounds of targeted rotations before falling back to sweeps

template <typename T>
__device__ void js_offnorm(const T *A, int N, int LD, double *red, double &off, double &tot) {
  double o = 0, t = 0;
  for (int idx = threadIdx.x; idx < N * N; idx += blockDim.x) {
    const int i = idx % N, j = idx / N;
    const double a = (double)A[i + j * LD];
    t += a * a;
    if (i != j) o += a * a;
  }
  off = block_sum(o, red);
  tot = block_sum(t, red);
}

// Square root and absolute value in T's own precision (the float overloads must not widen to double).
__device__ __forceinline__ float js_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double js_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float js_abs(float x) { return fabsf(x); }
__device__ __forceinline__ double js_abs(double x) { return fabs(x); }

// Slot i of the circle method after r rounds: slot 0 holds element 0; slots 1..M-1 hold a rotation of
// elements 1..M-1 (one step per round), so after r rounds slot i holds ((i - 1 - r) mod (M-1)) + 1.
__device__ __forceinline__ int js_slot(int i, int r, int M) {
  if (i == 0) return 0;
  const int x = (i - 1 - r) % (M - 1);
  return (x < 0 ? x + (M - 1) : x) + 1;
}

template <typename T>
__device__ void js_apply(T *A, T *V, int N, int LD, int M, const T *s_cs, const T *s_sn, const int *s_p,
                         const int *s_q);

// One cyclic sweep (M-1 rounds of M/2 disjoint rotations, circle-method pairing) on A and V.  The pairs
// of round r are (slot m, slot M-1-m); the pairing is the global kernel's, computed in closed form.
template <typename T>
__device__ void js_sweep(T *A, T *V, int N, int LD, int M, int *s_order, double *s_cs_d, double *s_sn_d, int *s_p,
                         int *s_q) {
  const int tid = threadIdx.x;
  (void)s_order;
  // the rotation parameters stay in T: a double <-> float conversion per element would run on the FP64 pipe
  T *s_cs = (T *)s_cs_d, *s_sn = (T *)s_sn_d;
  for (int round = 0; round < M - 1; round++) {
    // pair m's parameters on warp m % 4 (spreads the FP64 square roots and divisions over the SM's
    // four schedulers)
    const int m = (tid & 31) * 4 + (tid >> 5);
    if (tid < 128 && m < M / 2) {
      int p = js_slot(m, round, M), q = js_slot(M - 1 - m, round, M);
      if (p > q) {
        const int t = p;
        p = q;
        q = t;
      }
      T cs = (T)1, sn = (T)0;
      if (q < N) {
        const T apq = A[p + q * LD];
        if (apq != (T)0) {
          const T app = A[p + p * LD], aqq = A[q + q * LD];
          const T theta = (aqq - app) / ((T)2 * apq);
          const T t = (theta >= (T)0 ? (T)1 : (T)-1) / (js_abs(theta) + js_sqrt(theta * theta + (T)1));
          cs = (T)1 / js_sqrt(t * t + (T)1);
          sn = t * cs;
        }
      }
      s_p[m] = p;
      s_q[m] = q;
      s_cs[m] = cs;
      s_sn[m] = sn;
    }
    __syncthreads();
    js_apply<T>(A, V, N, LD, M, s_cs, s_sn, s_p, s_q);
  }
}

// A <- J^T A J and V <- V J for the M/2 disjoint rotations (s_p[m], s_q[m], s_cs[m], s_sn[m]) that partition the
// indices 0..M-1, in one step: every 2 x 2 block (rows of pair m1, columns of pair m2) takes its column
// rotation and then its row rotation, the same operations in the same order as rotating all columns first and
// all rows after, without a barrier in between (the pairs partition the indices, so blocks are disjoint).  A
// pair whose second index is the padding index N (odd N) or whose sine is 0 is the identity.  Ends with a
// barrier.
template <typename T>
__device__ void js_apply(T *A, T *V, int N, int LD, int M, const T *s_cs, const T *s_sn, const int *s_p,
                         const int *s_q) {
  const int tid = threadIdx.x;
  {
    const int P = M / 2;
    for (int it = tid; it < P * P; it += blockDim.x) {
      const int m1 = it / P, m2 = it - m1 * P;
      const int p1 = s_p[m1], q1 = s_q[m1];
      const T c1 = s_cs[m1], s1 = s_sn[m1];
      const bool q1ok = q1 < N;
      {
        const int p2 = s_p[m2], q2 = s_q[m2];
        const T c2 = s_cs[m2], s2 = s_sn[m2];
        const bool q2ok = q2 < N;
        const T a = A[p1 + p2 * LD];
        const T b = q2ok ? A[p1 + q2 * LD] : (T)0;
        const T d = q1ok ? A[q1 + p2 * LD] : (T)0;
        const T e = (q1ok && q2ok) ? A[q1 + q2 * LD] : (T)0;
        T a1 = a, b1 = b, d1 = d, e1 = e;
        if (q2ok && s2 != (T)0) {  // columns p2, q2
          a1 = c2 * a - s2 * b;
          b1 = s2 * a + c2 * b;
          d1 = c2 * d - s2 * e;
          e1 = s2 * d + c2 * e;
        }
        T a2 = a1, b2 = b1, d2 = d1, e2 = e1;
        if (q1ok && s1 != (T)0) {  // rows p1, q1
          a2 = c1 * a1 - s1 * d1;
          d2 = s1 * a1 + c1 * d1;
          b2 = c1 * b1 - s1 * e1;
          e2 = s1 * b1 + c1 * e1;
        }
        A[p1 + p2 * LD] = a2;
        if (q2ok) A[p1 + q2 * LD] = b2;
        if (q1ok) A[q1 + p2 * LD] = d2;
        if (q1ok && q2ok) A[q1 + q2 * LD] = e2;
      }
    }
    for (int idx = tid; idx < P * N; idx += blockDim.x) {
      const int m2 = idx / N, row = idx - m2 * N;
      const int p = s_p[m2], q = s_q[m2];
      const T cs = s_cs[m2], sn = s_sn[m2];
      if (q >= N || sn == (T)0) continue;
      const T vkp = V[row + p * LD], vkq = V[row + q * LD];
      V[row + p * LD] = cs * vkp - sn * vkq;
      V[row + q * LD] = sn * vkp + cs * vkq;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(EIG_THREADS) jacobi_smem_kernel(const double *Kin, int N, double *K, double *evals,
                                                                  int *sweeps, int *status, int max_sweeps,
                                                                  unsigned long long *trace, int c_target,
                                                                  int largest) {
#define JS_MARK(i)                                              \
  if (trace && blockIdx.x == 0 && threadIdx.x == 0) trace[i] = global_timer_ns();
  JS_MARK(0)
  extern __shared__ double js[];
  // a batch of problems: block b solves matrix b (N*N apart), with its own evals, sweeps and status
  Kin += (int64_t)blockIdx.x * N * N;
  K += (int64_t)blockIdx.x * N * N;
  evals += (int64_t)blockIdx.x * N;
  sweeps += blockIdx.x;
  status += blockIdx.x;
  // leading dimension LD = N | 1 (odd): the transposed accesses of a rotation's rows spread over all banks
  const int LD = N | 1;
  double *A = js, *V = js + N * LD, *W = js + 2 * N * LD;
  float *A32 = (float *)W, *V32 = (float *)W + N * LD;
  __shared__ double red[32];
  __shared__ double s_cs[JS_MAX_N / 2 + 1], s_sn[JS_MAX_N / 2 + 1];
  __shared__ int s_p[JS_MAX_N / 2 + 1], s_q[JS_MAX_N / 2 + 1];
  __shared__ int s_order[JS_MAX_N + 1];
  __shared__ int s_done;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int M = (N + 1) & ~1;
  for (int idx = tid; idx < N * N; idx += blockDim.x) {
    const int i = idx % N, j = idx / N;
    const double a = 0.5 * (Kin[i + j * N] + Kin[j + i * N]);
    A[i + j * LD] = a;
    A32[i + j * LD] = (float)a;
    V32[i + j * LD] = i == j ? 1.f : 0.f;
  }
  for (int i = tid; i < M; i += blockDim.x) s_order[i] = i;
  __syncthreads();
  // ---- FP32 sweeps: until FP32 rounding dominates the off-diagonal ----
  int sw32 = 0;
  double off = 0, tot = 0;
  for (; sw32 < 16; sw32++) {
    js_offnorm(A32, N, LD, red, off, tot);
    if (tid == 0) s_done = off <= 1e-11 * tot;
    __syncthreads();
    if (s_done) break;
    js_sweep<float>(A32, V32, N, LD, M, s_order, s_cs, s_sn, s_p, s_q);
  }
  JS_MARK(1)
  // ---- V = FP64 orthonormalisation of V32: V (V^T V)^(-1/2) to second order, V (I - E/2 + 3/8 E^2) with
  //      E = V^T V - I.  |E| is the rounding the FP32 rotations accumulated (~1e-5 at k = 64), so the first-order
  //      form would leave ~3/8 |E|^2 ~ 1e-10 in the eigenvalues; the neglected third-order term is ~1e-15 ----
  for (int idx = tid; idx < N * N; idx += blockDim.x) {
    const int i = idx % N, j = idx / N;
    V[i + j * LD] = (double)V32[i + j * LD];
  }
  __syncthreads();
  for (int idx = tid; idx < N * N; idx += blockDim.x) {  // W = E
    const int i = idx % N, j = idx / N;
    double e0 = 0, e1 = 0;
    int r = 0;
    for (; r + 1 < N; r += 2) {
      e0 = fma(V[r + i * LD], V[r + j * LD], e0);
      e1 = fma(V[r + 1 + i * LD], V[r + 1 + j * LD], e1);
    }
    if (r < N) e0 = fma(V[r + i * LD], V[r + j * LD], e0);
    W[i + j * LD] = (e0 + e1) - (i == j ? 1.0 : 0.0);
  }
  __syncthreads();
  {
    constexpr int PER = (JS_MAX_N * JS_MAX_N + JS_MIN_THREADS - 1) / JS_MIN_THREADS;
    double nv[PER];
    int cnt = 0;
    for (int idx = tid; idx < N * N; idx += blockDim.x, cnt++) {  // F = E/2 - 3/8 E^2, held until E is read
      const int i = idx % N, j = idx / N;
      double s0 = 0, s1 = 0;
      int l = 0;
      for (; l + 1 < N; l += 2) {
        s0 = fma(W[i + l * LD], W[l + j * LD], s0);
        s1 = fma(W[i + (l + 1) * LD], W[l + 1 + j * LD], s1);
      }
      if (l < N) s0 = fma(W[i + l * LD], W[l + j * LD], s0);
      nv[cnt] = 0.5 * W[i + j * LD] - 0.375 * (s0 + s1);
    }
    __syncthreads();
    cnt = 0;
    for (int idx = tid; idx < N * N; idx += blockDim.x, cnt++) W[idx % N + (idx / N) * LD] = nv[cnt];
    __syncthreads();
    cnt = 0;
    for (int idx = tid; idx < N * N; idx += blockDim.x, cnt++) {  // V - V F, held until every read is done
      const int r = idx % N, j = idx / N;
      double s0 = 0, s1 = 0;
      int l = 0;
      for (; l + 1 < N; l += 2) {
        s0 = fma(V[r + l * LD], W[l + j * LD], s0);
        s1 = fma(V[r + (l + 1) * LD], W[l + 1 + j * LD], s1);
      }
      if (l < N) s0 = fma(V[r + l * LD], W[l + j * LD], s0);
      nv[cnt] = V[r + j * LD] - (s0 + s1);
    }
    __syncthreads();
    cnt = 0;
    for (int idx = tid; idx < N * N; idx += blockDim.x, cnt++) V[idx % N + (idx / N) * LD] = nv[cnt];
  }
  __syncthreads();
  JS_MARK(2)
  // ---- A <- V^T A V in FP64 (W = A V, then A = V^T W, symmetrised) ----
  for (int idx = tid; idx < N * N; idx += blockDim.x) {
    const int i = idx % N, j = idx / N;
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    int l = 0;
    for (; l + 3 < N; l += 4) {
      s0 = fma(A[i + l * LD], V[l + j * LD], s0);
      s1 = fma(A[i + (l + 1) * LD], V[l + 1 + j * LD], s1);
      s2 = fma(A[i + (l + 2) * LD], V[l + 2 + j * LD], s2);
      s3 = fma(A[i + (l + 3) * LD], V[l + 3 + j * LD], s3);
    }
    for (; l < N; l++) s0 = fma(A[i + l * LD], V[l + j * LD], s0);
    W[i + j * LD] = (s0 + s1) + (s2 + s3);
  }
  __syncthreads();
  for (int idx = tid; idx < N * N; idx += blockDim.x) {
    const int i = idx % N, j = idx / N;
    if (i > j) continue;
    double s0 = 0, s1 = 0, t0 = 0, t1 = 0;
    int l = 0;
    for (; l + 1 < N; l += 2) {
      s0 = fma(V[l + i * LD], W[l + j * LD], s0);
      s1 = fma(V[l + 1 + i * LD], W[l + 1 + j * LD], s1);
      t0 = fma(V[l + j * LD], W[l + i * LD], t0);
      t1 = fma(V[l + 1 + j * LD], W[l + 1 + i * LD], t1);
    }
    if (l < N) {
      s0 = fma(V[l + i * LD], W[l + j * LD], s0);
      t0 = fma(V[l + j * LD], W[l + i * LD], t0);
    }
    const double s = 0.5 * ((s0 + s1) + (t0 + t1));
    // A is read by the W pass only, which finished at the barrier above
    A[i + j * LD] = s;
    A[j + i * LD] = s;
  }
  for (int i = tid; i < M; i += blockDim.x) s_order[i] = i;
  __syncthreads();
  JS_MARK(3)
  // ---- FP64 refinement.  A = V^T A V is exactly similar and off-diagonal to FP32 rounding.  When every
  //      pair is well separated (|a_ij| <= 1e-3 |a_ii - a_jj|), perturbation theory finishes the job:
  //      eigenvalues a_ii + sum_j a_ij^2 / (a_ii - a_jj) (error ~ off^3 / gap^2), eigenvectors e_i +
  //      sum_j a_ji / (lambda_i - a_jj) e_j, and for the c wanted ones two more fixed-point steps of
  //      (A - lambda_i) y = 0 with y_i = 1 (each gains a factor ~ off / gap).  Otherwise FP64 Jacobi
  //      sweeps. ----
  //      When some pairs are not separated (close eigenvalues) but none of them involves a wanted index (the
  //      c smallest or largest diagonal entries), FP64 rotations of just those pairs come first -- a few
  //      rounds of disjoint rotations, each as cheap as one round of a sweep, until every coupling left is
  //      either separated or negligible (1e-15 of the Frobenius norm) -- and the refinement then treats the
  //      negligible couplings of unseparated pairs as zero.  The wanted eigenpairs only ever divide by the
  //      gaps to separated eigenvalues.
  __shared__ double s_lam[JS_MAX_N];
  __shared__ int s_bad, s_full, s_nbad, s_nsel;
  __shared__ int s_cnt[JS_MAX_N + 1];
  __shared__ unsigned char s_want[JS_MAX_N + 1];
  __shared__ short s_bp[JS_BAD_CAP], s_bq[JS_BAD_CAP];
  if (tid == 0) {
    s_bad = 0;
    s_full = c_target * N > 2 * (int)blockDim.x;  // two refined entries per thread at most
  }
  __syncthreads();
  for (int idx = tid; idx < N * N; idx += blockDim.x) {
    const int i = idx % N, j = idx / N;
    if (i < j && !(fabs(A[i + j * LD]) <= 1e-3 * fabs(A[i + i * LD] - A[j + j * LD]))) s_bad = 1;
  }
  __syncthreads();
  int tj_rounds = 0;
  if (s_bad && !s_full) {
    js_offnorm(A, N, LD, red, off, tot);
    const double negl = 1e-15 * sqrt(tot);
    for (int i = tid; i < N; i += blockDim.x) {
      const double ai = A[i + i * LD];
      int rank = 0;
      for (int j = 0; j < N; j++) {
        const double aj = A[j + j * LD];
        rank += (aj < ai) || (aj == ai && j < i);
      }
      s_want[i] = largest ? rank >= N - c_target : rank < c_target;
    }
    __syncthreads();
    // pair (i, j), i < j: 0 separated or negligible, 1 to rotate, 2 unseparated with a wanted index
    auto pair_kind = [&](int i, int j) -> int {
      const double aij = A[i + j * LD], gap = fabs(A[i + i * LD] - A[j + j * LD]);
      const bool sep = fabs(aij) <= 1e-3 * gap;
      if (s_want[i] || s_want[j]) return (sep && gap > 0.0) ? 0 : 2;
      return (!sep && fabs(aij) > negl) ? 1 : 0;
    };
    for (;; tj_rounds++) {
      for (int i = tid; i < N; i += blockDim.x) {
        int cnt = 0;
        bool fb = false;
        for (int j = i + 1; j < N; j++) {
          const int kd = pair_kind(i, j);
          cnt += kd == 1;
          fb |= kd == 2;
        }
        s_cnt[i] = cnt;
        if (fb) s_full = 1;
      }
      __syncthreads();
      if (tid == 0) {
        int run = 0;
        for (int i = 0; i < N; i++) {
          const int c = s_cnt[i];
          s_cnt[i] = run;
          run += c;
        }
        s_nbad = run;
        if (run > JS_BAD_CAP || (run > 0 && tj_rounds == JS_TJ_MAX_ROUNDS)) s_full = 1;
      }
      __syncthreads();
      const int nbad = s_nbad;
      if (s_full || nbad == 0) break;  // uniform
      for (int i = tid; i < N; i += blockDim.x) {  // the pairs to rotate, in row order
        int pos = s_cnt[i];
        for (int j = i + 1; j < N; j++)
          if (pair_kind(i, j) == 1) {
            s_bp[pos] = (short)i;
            s_bq[pos] = (short)j;
            pos++;
          }
      }
      __syncthreads();
      if (tid == 0) {
        // greedy disjoint selection in list order; every other index (and the padding index N when N is odd)
        // goes into identity pairs, so the pairs partition 0..M-1 as js_apply expects
        for (int i = 0; i < N; i++) s_want[i] &= 1u;  // bit 1: taken this round
        int m = 0;
        for (int b = 0; b < nbad; b++) {
          const int p = s_bp[b], q = s_bq[b];
          if ((s_want[p] | s_want[q]) & 2u) continue;
          s_want[p] |= 2u;
          s_want[q] |= 2u;
          s_p[m] = p;
          s_q[m] = q;
          m++;
        }
        s_nsel = m;
        int prev = -1;
        for (int i = 0; i < M; i++) {
          if (i < N && (s_want[i] & 2u)) continue;
          if (prev < 0) {
            prev = i;
          } else {
            s_p[m] = prev;
            s_q[m] = i;
            s_cs[m] = 1.0;
            s_sn[m] = 0.0;
            m++;
            prev = -1;
          }
        }
        for (int i = 0; i < N; i++) s_want[i] &= 1u;
      }
      __syncthreads();
      for (int m = tid; m < s_nsel; m += blockDim.x) {
        const int p = s_p[m], q = s_q[m];
        const double apq = A[p + q * LD], app = A[p + p * LD], aqq = A[q + q * LD];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double cs = 1.0 / sqrt(t * t + 1.0);
        s_cs[m] = cs;
        s_sn[m] = t * cs;
      }
      __syncthreads();
      js_apply<double>(A, V, N, LD, M, s_cs, s_sn, s_p, s_q);
    }
  }
  int sw64 = 0;
  const double *Vout = V;  // eigenvector columns (unsorted), V itself after sweeps
  if (!s_full) {
    // (the separation test skips only the negligible couplings the targeted rotations left; with no
    // unseparated pair it never fails)
    for (int i = tid; i < N; i += blockDim.x) {
      const double aii = A[i + i * LD];
      double l0 = 0, l1 = 0;
      for (int j = 0; j < N; j++) {
        if (j == i) continue;
        const double aij = A[i + j * LD], ajj = A[j + j * LD];
        if (aij == 0.0 || !(fabs(aij) <= 1e-3 * fabs(aii - ajj))) continue;
        const double t = aij * aij / (aii - ajj);
        if (j & 1) l1 += t; else l0 += t;
      }
      s_lam[i] = aii + (l0 + l1);
    }
    __syncthreads();
    for (int idx = tid; idx < N * N; idx += blockDim.x) {  // W[:, i] = y_i to first order
      const int j = idx % N, i = idx / N;
      const double aji = A[j + i * LD], ajj = A[j + j * LD];
      W[j + i * LD] = j == i ? 1.0
                             : (aji != 0.0 && fabs(aji) <= 1e-3 * fabs(A[i + i * LD] - ajj) ? aji / (s_lam[i] - ajj)
                                                                                          : 0.0);
    }
    __syncthreads();
    // ranks of the eigenvalues: the wanted columns are the c smallest (or largest)
    for (int i = tid; i < N; i += blockDim.x) {
      const double li = s_lam[i];
      int rank = 0;
      for (int j = 0; j < N; j++) {
        const double lj = s_lam[j];
        rank += (lj < li) || (lj == li && j < i);
      }
      s_order[rank] = i;
    }
    __syncthreads();
    for (int it = 0; it < 2; it++) {
      // new y_j for j != i from the current y (computed into registers, written after a barrier)
      double ny[2];  // N * c_target <= 2 * blockDim.x (checked above)
      int cnt = 0;
      for (int idx = tid; idx < N * c_target; idx += blockDim.x, cnt++) {
        const int j = idx % N, ti = idx / N;
        const int i = s_order[largest ? N - 1 - ti : ti];
        double v = 1.0;
        if (j != i) {
          double s0 = 0, s1 = 0;
          for (int l = 0; l < N; l++) {
            if (l == j) continue;
            const double t = A[j + l * LD] * W[l + i * LD];
            if (l & 1) s1 += t; else s0 += t;
          }
          v = -(s0 + s1) / (A[j + j * LD] - s_lam[i]);
        }
        ny[cnt] = v;
      }
      __syncthreads();
      cnt = 0;
      for (int idx = tid; idx < N * c_target; idx += blockDim.x, cnt++) {
        const int j = idx % N, ti = idx / N;
        const int i = s_order[largest ? N - 1 - ti : ti];
        W[j + i * LD] = ny[cnt];
      }
      __syncthreads();
      for (int ti = tid; ti < c_target; ti += blockDim.x) {  // lambda_i = a_ii + sum_{l != i} a_il y_l
        const int i = s_order[largest ? N - 1 - ti : ti];
        double s0 = 0;
        for (int l = 0; l < N; l++)
          if (l != i) s0 = fma(A[i + l * LD], W[l + i * LD], s0);
        s_lam[i] = A[i + i * LD] + s0;
      }
      __syncthreads();
    }
    // eigenvectors of the original matrix: V y_i, normalised (A is no longer needed: it takes them)
    for (int idx = tid; idx < N * N; idx += blockDim.x) {
      const int r = idx % N, i = idx / N;
      double s0 = 0, s1 = 0;
      int l = 0;
      for (; l + 1 < N; l += 2) {
        s0 = fma(V[r + l * LD], W[l + i * LD], s0);
        s1 = fma(V[r + (l + 1) * LD], W[l + 1 + i * LD], s1);
      }
      if (l < N) s0 = fma(V[r + l * LD], W[l + i * LD], s0);
      A[r + i * LD] = s0 + s1;
    }
    __syncthreads();
    for (int i = warp; i < N; i += nw) {
      double d = 0;
      for (int r = lane; r < N; r += 32) d = fma(A[r + i * LD], A[r + i * LD], d);
      d = warp_sum(d);
      const double inv = 1.0 / sqrt(d);
      for (int r = lane; r < N; r += 32) A[r + i * LD] *= inv;
    }
    __syncthreads();
    Vout = A;
    off = 0;
    tot = 1;
  } else {
    for (; sw64 < max_sweeps; sw64++) {
      js_offnorm(A, N, LD, red, off, tot);
      if (tid == 0) s_done = (off <= 1e-24 * tot) || off == 0.0;
      __syncthreads();
      if (s_done) break;
      js_sweep<double>(A, V, N, LD, M, s_order, s_cs, s_sn, s_p, s_q);
    }
    if (sw64 == max_sweeps) js_offnorm(A, N, LD, red, off, tot);
    for (int i = tid; i < N; i += blockDim.x) s_lam[i] = A[i + i * LD];
    __syncthreads();
  }
  JS_MARK(4)
  if (trace && blockIdx.x == 0 && threadIdx.x == 0) {
    trace[6] = sw32;
    trace[7] = s_full ? sw64 : 1000 + tj_rounds;  // 1000 + r: refined by perturbation after r targeted rounds
  }
  // ascending order of the eigenvalues, ties by index (the stable order): rank of each entry, in parallel
  for (int i = tid; i < N; i += blockDim.x) {
    const double li = s_lam[i];
    int rank = 0;
    for (int j = 0; j < N; j++) {
      const double lj = s_lam[j];
      rank += (lj < li) || (lj == li && j < i);
    }
    s_order[rank] = i;
    evals[rank] = li;
  }
  if (tid == 0) {
    *sweeps = sw32 + sw64;
    *status = (sw64 < max_sweeps || off <= 1e-20 * tot) ? PHDE_OK : PHDE_ERR_NOCONVERGE;
  }
  __syncthreads();
  for (int c = warp; c < N; c += nw) {
    const int src = s_order[c];
    double best = -1.0;
    int arg = 0;
    for (int i = lane; i < N; i += 32) {
      const double a = fabs(Vout[i + src * LD]);
      if (a > best) {
        best = a;
        arg = i;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double b2 = __shfl_xor_sync(PHDE_FULL_MASK, best, o);
      const int a2 = __shfl_xor_sync(PHDE_FULL_MASK, arg, o);
      if (b2 > best || (b2 == best && a2 < arg)) {
        best = b2;
        arg = a2;
      }
    }
    const double sg = Vout[arg + src * LD] < 0 ? -1.0 : 1.0;
    for (int i = lane; i < N; i += 32) K[i + c * N] = sg * Vout[i + src * LD];
  }
  __syncthreads();
  JS_MARK(5)
#undef JS_MARK
}

__global__ void pick_kernel(const double *K, int N, int c, int largest, double *Y) {
  K += (int64_t)blockIdx.x * N * N;  // batch: block b picks from matrix b
  Y += (int64_t)blockIdx.x * N * c;
  for (int idx = threadIdx.x; idx < N * c; idx += blockDim.x) {
    const int i = idx % N, j = idx / N;
    const int col = largest ? N - 1 - j : j;
    Y[idx] = K[i + col * N];
  }
}

// Threads of the shared-memory solver: its rounds are barrier bound, so the fewest that still cover a
// round's work (measured on GB300: 256 up to N = 16, 512 above).  PHDE_JACOBI_THREADS overrides.
int js_threads(int N) {
  if (const char *e = getenv("PHDE_JACOBI_THREADS")) {
    const int t = atoi(e);
    if (t == 256 || t == 512 || t == 1024) return t;
  }
  return N <= 16 ? 256 : 512;
}

}  // namespace

// Solve the k x k problem in d_M (column-major).  On success d_K holds the eigenvector matrix,
// d_evals the eigenvalues (ascending), d_Y the c picked eigenvectors.  Synchronises to read the status.
int phde_eigensolve(phde_ctx *ctx, const double *d_M, int N, int c, int largest, int eig, double *d_K,
                    double *d_evals, double *d_Y, int *h_iters, int seq) {
  double *w1 = (double *)phde_buf(ctx, "eig.w1", sizeof(double) * N * N);
  double *w2 = (double *)phde_buf(ctx, "eig.w2", sizeof(double) * N * N);
  double *dd = (double *)phde_buf(ctx, "eig.dd", sizeof(double) * N);
  int *st = (int *)phde_buf(ctx, "eig.st", sizeof(int) * 2);
  if (!w1 || !w2 || !dd || !st) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemsetAsync(st, 0, sizeof(int) * 2, ctx->stream));
  if (eig == PHDE_EIG_EXACT) {
    if (N <= JS_MAX_N && !getenv("PHDE_JACOBI_GLOBAL")) {
      const size_t jsmem = sizeof(double) * 3 * (size_t)N * (N | 1);
      PHDE_CK(ctx, cudaFuncSetAttribute(jacobi_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)jsmem));
      // PHDE_EIG_TRACE=1: print the kernel's phase timeline (FP32 sweeps, orthonormalisation, similarity,
      // FP64 sweeps, sort) after the solve
      unsigned long long *tr = getenv("PHDE_EIG_TRACE") ? (unsigned long long *)phde_buf(ctx, "eig.trace", 64) : nullptr;
      jacobi_smem_kernel<<<1, js_threads(N), jsmem, ctx->stream>>>(d_M, N, d_K, d_evals, st, st + 1, 100, tr, c,
                                                                    largest);
      if (tr) {
        unsigned long long h[8];
        PHDE_CK(ctx, cudaMemcpyAsync(h, tr, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
        PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
        fprintf(stderr, "jacobi N=%d: fp32 sweeps %llu: %.1f us, orthonormalise %.1f us, similarity %.1f us, "
                        "fp64 sweeps %llu (1000 + r: refined after r targeted rounds): %.1f us, sort/sign %.1f us\n", N, h[6], (h[1] - h[0]) * 1e-3,
                (h[2] - h[1]) * 1e-3, (h[3] - h[2]) * 1e-3, h[7], (h[4] - h[3]) * 1e-3, (h[5] - h[4]) * 1e-3);
      }
    } else {
      jacobi_kernel<<<1, EIG_THREADS, 0, ctx->stream>>>(d_M, N, w1, w2, d_K, d_evals, st, st + 1, 100);
    }
  } else {
    const int NO = (N + PW_CL - 1) / PW_CL;
    const size_t csmem = sizeof(double) * ((size_t)N * N + 2 * (size_t)NO * N + 2 * NO + 1);
    if (seq || N > PW_MAX_N || getenv("PHDE_POWER_SINGLE_CTA")) {
      if (seq)
        power_kernel<true><<<1, EIG_THREADS, 0, ctx->stream>>>(d_M, N, d_K, w1, w2, d_evals, st, st + 1, 20000, dd);
      else
        power_kernel<false><<<1, EIG_THREADS, 0, ctx->stream>>>(d_M, N, d_K, w1, w2, d_evals, st, st + 1, 20000, dd);
    } else {
      PHDE_CK(ctx, cudaFuncSetAttribute(power_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csmem));
      power_cluster_kernel<<<PW_CL, EIG_THREADS, csmem, ctx->stream>>>(d_M, N, d_K, d_evals, st, st + 1, 20000);
    }
  }
  PHDE_LAUNCHED(ctx);
  pick_kernel<<<1, 256, 0, ctx->stream>>>(d_K, N, c, largest, d_Y);
  PHDE_LAUNCHED(ctx);
  int h[2];
  PHDE_CK(ctx, cudaMemcpyAsync(h, st, sizeof(int) * 2, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  *h_iters = h[0];
  if (h[1] != PHDE_OK)
    return phde_fail(ctx, h[1], eig == PHDE_EIG_EXACT ? "Jacobi eigensolver did not converge"
                                                      : "power iteration did not converge (iteration cap reached)");
  return PHDE_OK;
}

// Batched exact solve: `count` k x k problems (column-major, N*N apart) in one launch, one CTA each
// (shared-memory Jacobi; N <= JS_MAX_N).  d_st holds 2*count ints (sweeps, status).  No synchronisation:
// the caller reads d_st when it next synchronises.
int phde_eigensolve_batched(phde_ctx *ctx, const double *d_M, int N, int c, int count, double *d_K,
                            double *d_evals, double *d_Y, int *d_st) {
  if (N > JS_MAX_N) return phde_fail(ctx, PHDE_ERR_INVALID, "batched eigensolve: k above the shared-memory limit");
  const size_t jsmem = sizeof(double) * 3 * (size_t)N * (N | 1);
  PHDE_CK(ctx, cudaFuncSetAttribute(jacobi_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)jsmem));
  jacobi_smem_kernel<<<count, js_threads(N), jsmem, ctx->stream>>>(d_M, N, d_K, d_evals, d_st, d_st + count, 100,
                                                                    nullptr, c, 0);
  PHDE_LAUNCHED(ctx);
  pick_kernel<<<count, 256, 0, ctx->stream>>>(d_K, N, c, 0, d_Y);
  PHDE_LAUNCHED(ctx);
  return PHDE_OK;
}

// Diagnostics entry: the exact (Jacobi) eigensolver of the layouts on a caller's symmetric k x k matrix.
extern "C" int phde_symeig(phde_ctx *ctx, const double *M, int k, int c, int largest, double *evals, double *Y,
                           int *iters) {
  if (!ctx) return PHDE_ERR_INVALID;
  if (!M || !evals || !Y || k < 1 || k > PHDE_MAX_K || c < 1 || c > k)
    return phde_fail(ctx, PHDE_ERR_INVALID, "phde_symeig: bad arguments");
  PHDE_CK(ctx, cudaSetDevice(ctx->device));
  double *dM = (double *)phde_buf(ctx, "symeig.M", sizeof(double) * k * k);
  double *dK = (double *)phde_buf(ctx, "symeig.K", sizeof(double) * k * k);
  double *dE = (double *)phde_buf(ctx, "symeig.E", sizeof(double) * k);
  double *dY = (double *)phde_buf(ctx, "symeig.Y", sizeof(double) * k * c);
  if (!dM || !dK || !dE || !dY) return PHDE_ERR_OOM;
  PHDE_CK(ctx, cudaMemcpyAsync(dM, M, sizeof(double) * k * k, cudaMemcpyHostToDevice, ctx->stream));
  int it = 0;
  int rc = phde_eigensolve(ctx, dM, k, c, largest ? 1 : 0, PHDE_EIG_EXACT, dK, dE, dY, &it, 0);
  if (rc) return rc;
  PHDE_CK(ctx, cudaMemcpyAsync(evals, dE, sizeof(double) * k, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaMemcpyAsync(Y, dY, sizeof(double) * k * c, cudaMemcpyDeviceToHost, ctx->stream));
  PHDE_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (iters) *iters = it;
  return PHDE_OK;
}
