// bcgs_gs.cuh -- the accept/discard loop of blocked CGS2 in the block's coefficient space (FP64).
//
// For a block of up to 32 candidates X (already projected twice against the accepted basis), with the
// block Gram matrices Gd = X^T D X and G2 = X^T X, candidate i is t = e_i in coefficient space; it is
// projected twice against the block's accepted vectors r_a (c_a = t^T Gd r_a / r_a^T Gd r_a, all from the
// same t: classical Gram-Schmidt, ParHDE.cpp:190-285), its norm is sqrt(t^T G2 t), and it is discarded
// below 1e-3 (ParHDE.cpp:267) or accepted as r = t / norm (ParHDE.cpp:270-276), until k are accepted.
//
// GB300 issues FP64 at 1/64 of its FP32 rate, so the cost is the number of FP64 warp instructions: every
// 32-term product is split over the four warps of the CTA (one per SM sub-partition), eight terms each,
// and the partial sums meet in shared memory.  Lane m of every warp holds component m of t.  The first
// projection pass starts from t = e_i, where <t, Gd r_a> is the stored (Gd r_a)[i]: no product at all.
#pragma once
#include "common.cuh"

namespace bcgs_gs {

constexpr int BB = 32;
constexpr int NW = 4;  // warps; the CTA has NW * 32 threads

struct Smem {
  double Gd[BB][BB + 1], G2[BB][BB + 1];
  double R[BB][BB + 1];  // R[a][m]: accepted vector a
  double U[BB][BB + 1];  // U[a][m] = (Gd r_a)[m]
  double dd[BB];         // r_a^T Gd r_a
  double tv[BB];
  double part[NW][BB];
  double cv[BB];
};

// sum over l in warp w's quarter of M[row][l] * v[l]
__device__ __forceinline__ double quarter_dot(const double (*M)[BB + 1], int row, const double *v, int w) {
  const int l0 = w * (BB / NW);
  double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
#pragma unroll
  for (int l = 0; l < BB / NW; l += 4) {
    a0 = fma(M[row][l0 + l], v[l0 + l], a0);
    a1 = fma(M[row][l0 + l + 1], v[l0 + l + 1], a1);
    a2 = fma(M[row][l0 + l + 2], v[l0 + l + 2], a2);
    a3 = fma(M[row][l0 + l + 3], v[l0 + l + 3], a3);
  }
  return (a0 + a1) + (a2 + a3);
}

// Runs the loop for one block; Gd/G2 are 32 x 32 row-major FP64 in global memory.  j0 = accepted so far.
// Writes R (32 x 32 FP32, R[i * 32 + a] = component i of accepted vector a) and dlog[i] for discarded
// candidates; returns (in thread 0's outputs) the counts.  Every thread of the CTA must call it.
__device__ __forceinline__ void run(Smem &S, const double *Gd, const double *G2, int bc, int k, int j0,
                                    double *dlog, float *R, int *nacc_out, int *ndisc_out, int *ncons_out) {
  const int m = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int idx = threadIdx.x; idx < BB * BB; idx += NW * 32) {
    S.Gd[idx / BB][idx % BB] = Gd[idx];
    S.G2[idx / BB][idx % BB] = G2[idx];
  }
  __syncthreads();
  int nacc = 0, ndisc = 0, ncons = 0;
  for (int i = 0; i < bc; i++) {
    if (j0 + nacc >= k) break;
    ncons++;
    double t = m == i ? 1.0 : 0.0;  // every warp keeps the same t
    for (int pass = 0; pass < 2 && nacc > 0; pass++) {
      if (pass == 0) {
        // t = e_i: <t, U_a> is U_a[i] exactly, no dot product needed
        if (w == 0 && m < nacc) S.cv[m] = S.U[m][i] / S.dd[m];
      } else {
        if (w == 0) S.tv[m] = t;
        __syncthreads();
        // c_a = <t, U_a> / dd_a (lane a), each warp a quarter of the terms
        S.part[w][m] = m < nacc ? quarter_dot(S.U, m, S.tv, w) : 0.0;
        __syncthreads();
        if (w == 0 && m < nacc) S.cv[m] = ((S.part[0][m] + S.part[1][m]) + (S.part[2][m] + S.part[3][m])) / S.dd[m];
      }
      __syncthreads();
      // t -= sum_a c_a R[a][m], warp w takes a = w, w + 4, ...
      double s = 0;
      for (int a = w; a < nacc; a += NW) s = fma(S.cv[a], S.R[a][m], s);
      S.part[w][m] = s;
      __syncthreads();
      t -= (S.part[0][m] + S.part[1][m]) + (S.part[2][m] + S.part[3][m]);
      __syncthreads();
    }
    if (w == 0) S.tv[m] = t;
    __syncthreads();
    S.part[w][m] = quarter_dot(S.G2, m, S.tv, w);  // (G2 t)[m]
    __syncthreads();
    const double g = (S.part[0][m] + S.part[1][m]) + (S.part[2][m] + S.part[3][m]);
    const double nrm = sqrt(fmax(warp_sum(t * g), 0.0));
    __syncthreads();
    if (nrm < 0.001) {
      ndisc++;
      if (threadIdx.x == 0) dlog[i] = nrm;
    } else {
      const double r = t / nrm;
      if (w == 0) S.tv[m] = r;
      __syncthreads();
      S.part[w][m] = quarter_dot(S.Gd, m, S.tv, w);  // (Gd r)[m]
      __syncthreads();
      const double u = (S.part[0][m] + S.part[1][m]) + (S.part[2][m] + S.part[3][m]);
      const double d = warp_sum(r * u);
      if (w == 0) {
        S.R[nacc][m] = r;
        S.U[nacc][m] = u;
        if (m == 0) S.dd[nacc] = d;
      }
      nacc++;
      __syncthreads();
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
