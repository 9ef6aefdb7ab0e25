// bcgs_gs.cuh -- the accept/discard loop of blocked CGS2 in the block's coefficient space (FP64).
//
// For a block of up to 32 candidates X (already projected twice against the accepted basis), with the
// block Gram matrices Gd = X^T D X and G2 = X^T X, candidate i is t = e_i in coefficient space; it is
// projected twice against the block's accepted vectors r_a (c_a = t^T Gd r_a / r_a^T Gd r_a, all from the
// same t: classical Gram-Schmidt, ParHDE.cpp:190-285), its norm is sqrt(t^T G2 t), and it is discarded
// below 1e-3 (ParHDE.cpp:267) or accepted as r = t / norm (ParHDE.cpp:270-276), until k are accepted.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, so every 32-term product is split over the four warps of
// the CTA (one per SM sub-partition, each with its own FP64 unit), eight terms each.  The first projection
// pass starts from t = e_i, where <t, Gd r_a> is the stored (Gd r_a)[i]: no product at all; divisions by
// r_a^T Gd r_a are multiplications by its stored reciprocal.
#pragma once
#include "common.cuh"

namespace bcgs_gs {

constexpr int BB = 32;
constexpr int NW = 4;  // warps; the CTA has NW * 32 threads

struct Smem {
  double Gd[BB][BB + 1], G2[BB][BB + 1];
  double R[BB][BB + 1];  // R[a][m]: accepted vector a
  double U[BB][BB + 1];  // U[a][m] = (Gd r_a)[m]
  double rdd[BB];        // 1 / (r_a^T Gd r_a)
  double part[2][NW][BB];  // per-warp partial sums, two buffers used in turn
};

// sum over l in warp w's quarter of M[row][l] * x_l, where lane l of the calling warp holds x_l
__device__ __forceinline__ double quarter_dot(const double (*M)[BB + 1], int row, double x, int w) {
  const int l0 = w * (BB / NW);
  double a0 = 0, a1 = 0;
#pragma unroll
  for (int l = 0; l < BB / NW; l += 2) {
    a0 = fma(M[row][l0 + l], __shfl_sync(PHDE_FULL_MASK, x, l0 + l), a0);
    a1 = fma(M[row][l0 + l + 1], __shfl_sync(PHDE_FULL_MASK, x, l0 + l + 1), a1);
  }
  return a0 + a1;
}

// sum over a < nacc with a = w mod NW of c_a * R[a][m], where lane a holds c_a
__device__ __forceinline__ double strided_combine(const double (*Rm)[BB + 1], int nacc, int m, double c, int w) {
  double s = 0;
  for (int a = w; a < nacc; a += NW) s = fma(__shfl_sync(PHDE_FULL_MASK, c, a), Rm[a][m], s);
  return s;
}

// Runs the loop for one block; Gd/G2 are 32 x 32 row-major FP64 in global memory.  j0 = accepted so far.
// Writes R (32 x 32 FP32, R[i * 32 + a] = component i of accepted vector a) and dlog[i] for discarded
// candidates; returns (in thread 0's outputs) the counts.  Every thread of the CTA must call it.
//
// Every warp keeps the whole candidate t (lane m: component m), so a product's quarter reads t by shuffle;
// the four quarters meet in shared memory with one barrier per product (two partial-sum buffers used in
// turn, so the next product may be written while a slower warp still reads the last), and every warp then
// forms the same sum in the same order.
__device__ __forceinline__ void run(Smem &S, const double *Gd, const double *G2, int bc, int k, int j0,
                                    double *dlog, float *R, int *nacc_out, int *ndisc_out, int *ncons_out) {
  const int m = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int idx = threadIdx.x; idx < BB * BB; idx += NW * 32) {
    S.Gd[idx / BB][idx % BB] = Gd[idx];
    S.G2[idx / BB][idx % BB] = G2[idx];
  }
  __syncthreads();
  int buf = 0;
  // one product's four quarters summed: write, barrier, add in warp order
  auto meet = [&](double mine) -> double {
    S.part[buf][w][m] = mine;
    __syncthreads();
    const double r = (S.part[buf][0][m] + S.part[buf][1][m]) + (S.part[buf][2][m] + S.part[buf][3][m]);
    buf ^= 1;
    return r;
  };
  int nacc = 0, ndisc = 0, ncons = 0;
  for (int i = 0; i < bc; i++) {
    if (j0 + nacc >= k) break;
    ncons++;
    double t = m == i ? 1.0 : 0.0;
    if (nacc > 0) {
      // pass 1 from t = e_i: <t, Gd r_a> is the stored (Gd r_a)[i]
      double c = m < nacc ? S.U[m][i] * S.rdd[m] : 0.0;
      t -= meet(strided_combine(S.R, nacc, m, c, w));
      // pass 2: c_a = <t, Gd r_a> / dd_a (lane a), then t -= sum_a c_a r_a
      const double p = meet(quarter_dot(S.U, m < nacc ? m : 0, t, w));
      c = m < nacc ? p * S.rdd[m] : 0.0;
      t -= meet(strided_combine(S.R, nacc, m, c, w));
    }
    const double g = meet(quarter_dot(S.G2, m, t, w));  // (G2 t)[m]
    const double nrm = sqrt(fmax(warp_sum(t * g), 0.0));
    if (nrm < 0.001) {
      ndisc++;
      if (threadIdx.x == 0) dlog[i] = nrm;
    } else {
      const double r = t / nrm;
      const double u = meet(quarter_dot(S.Gd, m, r, w));  // (Gd r)[m]
      const double d = warp_sum(r * u);
      if (w == 0) {
        S.R[nacc][m] = r;
        S.U[nacc][m] = u;
        if (m == 0) S.rdd[nacc] = 1.0 / d;
      }
      nacc++;
      __syncthreads();  // the new vector is visible to every warp before the next candidate reads it
    }
  }
  for (int idx = threadIdx.x; idx < BB * BB; idx += NW * 32) {
    const int row = idx / BB, a = idx % BB;  // R[row * 32 + a] = component row of vector a
    R[idx] = a < nacc ? (float)S.R[a][row] : 0.f;
  }
  if (threadIdx.x == 0) {
    *nacc_out = nacc;
    *ndisc_out = ndisc;
    *ncons_out = ncons;
  }
}

}  // namespace bcgs_gs
