// PCR-pThomas pieces: the PCR steps (shared by the direct-load kernel,
// pcr.cu, and the persistent TMA-fed chunk kernel, wm.cu) and the
// one-chain-per-lane Thomas of the direct-load kernel.
//
// A warp holds one system of 32*Q rows, lane l the Q consecutive rows
// l*Q .. l*Q+Q-1 (identity rows past n).  Five PCR steps with strides 1, 2,
// 4, 8, 16 leave every row coupled only to the rows 32 above and below (four
// steps, for the half variant of wm.cu: 16 above and below); a step of
// stride s < Q finds most neighbours in the lane's own registers and
// exchanges only the s rows at each end of the chunk with the adjacent lane
// (6 s shuffles), strides s >= Q shift whole lanes (6 Q shuffles, or an
// exchange through shared memory).
//
// Chain transpose.  Afterwards chain c (rows c, c+32, ...) is solved by lane
// c.  The rows pass through shared memory at index
//     r -> 32 (r >> 5) + ((r & 31) ^ ((r >> 5) & 31))
// which is conflict-free both for the chunk-wise writes (lane l, row l*Q+q)
// and the chain-wise reads (lane c, row c + 32 k), with no padding.
#pragma once

#include "common.cuh"
#include "tw.cuh"

namespace tdg {

__device__ __forceinline__ int pcr_swz(int r) { return (r & ~31) | ((r & 31) ^ ((r >> 5) & 31)); }

// Whole-lane neighbour exchange for the PCR strides s >= Q: lo receives v of
// lane - ls, hi v of lane + ls.  Lanes whose partner lies outside the warp
// receive a finite value of their own warp, which reaches only rows whose
// coupling coefficient is an exact zero (see pcr_chunk_steps).
struct PcrShfl {
  template <typename T, int Q>
  __device__ __forceinline__ void lanes(const T (&v)[Q], T (&lo)[Q], T (&hi)[Q], int, int ls) const {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      lo[q] = shfl_up(v[q], ls);
      hi[q] = shfl_down(v[q], ls);
    }
  }
};

// STEPS PCR steps (strides 1 .. 2^(STEPS-1)) on the lane's chunk (A, B, C,
// D updated in place): five for PCR-pThomas (32 chains of stride 32), four
// for the half variant (16 chains of stride 16).
//
// Ends of the system.  A of row 0 and C of row 32 Q - 1 must be zero (the
// callers load them so; rows past n are identity rows, A = C = 0).  Step s
// then keeps A = 0 on rows < 2 s and C = 0 on rows >= 32 Q - 2 s (each new
// coefficient is a product with the old one or with the neighbour's), so a
// neighbour that lies outside the system is always multiplied by an exact
// zero: the exchanges take whatever finite value the shuffle returns there
// instead of selecting an identity row (one select per exchanged value).
template <typename T, int Q, int STEPS = 5, typename X = PcrShfl>
__device__ __forceinline__ void pcr_chunk_steps(T (&A)[Q], T (&B)[Q], T (&C)[Q], T (&D)[Q], int lane,
                                                const X& xch = X()) {
#pragma unroll
  for (int s = 1; s < (1 << STEPS); s <<= 1) {
    T al[Q], ga[Q], de[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const Div<T> k(B[q]);
      al[q] = k.div(A[q]);
      ga[q] = k.div(C[q]);
      de[q] = k.div(D[q]);
    }
    // neighbours s rows above (L) and below (R)
    T aL[Q], gL[Q], dL[Q], aR[Q], gR[Q], dR[Q];
    if (s < Q) {
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        if (q >= s) {
          aL[q] = al[q - s];
          gL[q] = ga[q - s];
          dL[q] = de[q - s];
        } else {  // row q - s + Q of lane - 1
          aL[q] = shfl_up(al[q - s + Q], 1);
          gL[q] = shfl_up(ga[q - s + Q], 1);
          dL[q] = shfl_up(de[q - s + Q], 1);
        }
        if (q + s < Q) {
          aR[q] = al[q + s];
          gR[q] = ga[q + s];
          dR[q] = de[q + s];
        } else {  // row q + s - Q of lane + 1
          aR[q] = shfl_down(al[q + s - Q], 1);
          gR[q] = shfl_down(ga[q + s - Q], 1);
          dR[q] = shfl_down(de[q + s - Q], 1);
        }
      }
    } else {
      const int ls = s / Q;  // whole lanes
      xch.lanes(al, aL, aR, lane, ls);
      xch.lanes(ga, gL, gR, lane, ls);
      xch.lanes(de, dL, dR, lane, ls);
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const T a0 = A[q], c0 = C[q];
      A[q] = -a0 * aL[q];
      B[q] = fma(-c0, aR[q], fma(-a0, gL[q], B[q]));
      C[q] = -c0 * gR[q];
      D[q] = fma(-c0, dR[q], fma(-a0, dL[q], D[q]));
    }
  }
}

// Normalise the lane's rows (unit diagonal), pass them through `scratch`
// (32*Q values, one array at a time) so that lane c holds chain c, and run
// Thomas on it.  Returns x of rows c + 32 k in X[k].  The caller's scratch
// must be free; it is left in use (no trailing sync).
template <typename T, int Q>
__device__ __forceinline__ void pcr_chain_thomas(T (&A)[Q], T (&B)[Q], T (&C)[Q], T (&D)[Q], T (&X)[Q], int lane,
                                                 T* scratch) {
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const Div<T> k(B[q]);
    A[q] = k.div(A[q]);
    C[q] = k.div(C[q]);
    D[q] = k.div(D[q]);
  }
  // chunk -> chain, one array per round (B receives the chain values of A,
  // then A of C, then C of D)
  T ca[Q], cg[Q], cd[Q];
#pragma unroll
  for (int round = 0; round < 3; ++round) {
#pragma unroll
    for (int q = 0; q < Q; ++q) scratch[pcr_swz(lane * Q + q)] = round == 0 ? A[q] : round == 1 ? C[q] : D[q];
    __syncwarp();
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      const T v = scratch[pcr_swz(lane + 32 * k)];
      if (round == 0) ca[k] = v;
      else if (round == 1) cg[k] = v;
      else cd[k] = v;
    }
    __syncwarp();
  }
  T cp = T(0), dp = T(0);
#pragma unroll
  for (int k = 0; k < Q; ++k) {
    const Div<T> den(fma(-ca[k], cp, T(1)));
    cp = den.div(cg[k]);
    dp = den.div(fma(-ca[k], dp, cd[k]));
    cg[k] = cp;
    cd[k] = dp;
  }
  T xv = T(0);
#pragma unroll
  for (int kk = 0; kk < Q; ++kk) {
    const int k = Q - 1 - kk;
    xv = fma(-cg[k], xv, cd[k]);
    X[k] = xv;
  }
}

}  // namespace tdg
