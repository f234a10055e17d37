// pgb_spmv.cuh -- the CSR-adaptive sparse matrix-vector core shared by the
// plain operator application and the fused Lanczos steps.
//
// Row blocks (built once per matrix) are either a run of short rows whose
// nonzeros fit the CTA's shared-memory stage, or one long row.  A run is
// streamed with fully coalesced loads of the column indices and values, the
// products val*x[col] are parked in shared memory, and every row is then
// summed by a group of g lanes (g = BS / rows in the block, a power of two
// <= 32).  A long row is reduced by the whole CTA.  Summation order depends
// only on the matrix, never on timing, so results are bit-reproducible.
#pragma once
#include "pgb.cuh"

namespace pgb {

// Shared-memory stage of one row block.
template <typename VT>
struct SpmvStage {
    int idx[NNZ_PB];
    VT val[NNZ_PB];
};

// visit every row owned by this CTA; epi(row, sum) is called by exactly one
// thread per row.  xload(col) returns the gathered input for a column.
// AT is the accumulation type (double for the FP64 path, float for FP32).
template <typename VT, typename AT, typename XF, typename EPI>
__device__ __forceinline__ void csr_rows(const int *__restrict__ ptr, const int *__restrict__ idx,
                                         const VT *__restrict__ val, const int *__restrict__ blk,
                                         int nblk, XF xload, EPI epi, SpmvStage<VT> &st, double *sred)
{
    const int tid = threadIdx.x;
    for (int b = blockIdx.x; b < nblk; b += gridDim.x) {
        const int r0 = blk[b], r1 = blk[b + 1];
        const int e0 = ptr[r0], e1 = ptr[r1];
        const int nr = r1 - r0;
        if (nr > 1) {
            // stage the block's column indices and values (coalesced)
            int e = e0 + tid;
            for (; e + 3 * BS < e1; e += 4 * BS) {
                const int c0 = idx[e], c1 = idx[e + BS], c2 = idx[e + 2 * BS], c3 = idx[e + 3 * BS];
                const VT v0 = val[e], v1 = val[e + BS], v2 = val[e + 2 * BS], v3 = val[e + 3 * BS];
                st.idx[e - e0] = c0; st.idx[e - e0 + BS] = c1;
                st.idx[e - e0 + 2 * BS] = c2; st.idx[e - e0 + 3 * BS] = c3;
                st.val[e - e0] = v0; st.val[e - e0 + BS] = v1;
                st.val[e - e0 + 2 * BS] = v2; st.val[e - e0 + 3 * BS] = v3;
            }
            for (; e < e1; e += BS) { st.idx[e - e0] = idx[e]; st.val[e - e0] = val[e]; }
            __syncthreads();
            // g lanes per row
            int g = 32;
            while (g > 1 && g * nr > BS) g >>= 1;
            const int grp = tid / g, lig = tid % g;
            const int ngrp = BS / g;
            // every lane runs the same number of rounds so the group
            // shuffles always see the full warp
            for (int base = r0; base < r1; base += ngrp) {
                const int r = base + grp;
                AT acc = 0;
                if (r < r1) {
                    const int a = ptr[r] - e0, z = ptr[r + 1] - e0;
                    for (int q = a + lig; q < z; q += g) acc = fma((AT)st.val[q], (AT)xload(st.idx[q]), acc);
                }
                for (int o = g >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, g);
                if (r < r1 && lig == 0) epi(r, (double)acc);
            }
            __syncthreads();
        } else if (nr == 1) {
            AT acc = 0;
            for (int e = e0 + tid; e < e1; e += BS) acc = fma((AT)val[e], (AT)xload(idx[e]), acc);
            const double t = block_sum<BS>((double)acc, sred);
            if (tid == 0) epi(r0, t);
        }
    }
}

}  // namespace pgb
