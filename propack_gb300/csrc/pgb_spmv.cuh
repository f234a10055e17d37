// pgb_spmv.cuh -- the CSR-stream sparse matrix-vector core shared by the
// plain operator application and the fused Lanczos steps.
//
// Row blocks (built once per matrix) hold at most ROWS_W rows and NNZ_W
// nonzeros, or one long row.  Each warp owns whole blocks and works without
// CTA barriers: every lane issues all of its (index, value) loads for the
// block, then all of its gathers x[index] (one HBM and one L2 round trip
// per block, many requests in flight), and parks value and gathered input
// in its warp's slice of shared memory.  g lanes per row (g = 32 / rows in
// the block, a power of two) then form the row sums from shared memory; with
// ~20-nonzero rows g is 1 or 2, so the FP64 pipe issues about one FMA per
// nonzero and almost no shuffle adds.  A long row is streamed by the whole
// warp straight from global memory.  Summation order depends only on the
// matrix, never on timing, so results are bit-reproducible.
#pragma once
#include "pgb.cuh"

namespace pgb {

constexpr int SPMV_WARPS = BS / 32;  // warps per CTA

// One warp's shared-memory stage: the block's values and gathered inputs.
template <typename VT, typename AT>
struct SpmvStage {
    VT val[NNZ_W];
    AT xv[NNZ_W];
};

constexpr int SPMV_PER_LANE = NNZ_W / 32;  // staged nonzeros per lane

// Visit every row; epi(row, sum, pre) is called by exactly one lane per row,
// where pre = pre_load(row) was issued early (with the block's own loads) so
// that per-row epilogue inputs never add a round trip.  xload(col) returns
// the gathered input for a column.  AT is the accumulation type (double for
// the FP64 path, float for FP32).
//
// Per block each lane issues, all at once, its (index, value) loads, the
// row pointer and the pre_load of "its" row (lane l owns row r0+l), and the
// bounds of the warp's next block; then all of its gathers.  So a block
// costs one HBM and one L2 round trip; the row sums read shared memory and
// row bounds / pre values arrive by warp shuffles.
template <typename VT, typename AT, typename XF, typename PF, typename EPI>
__device__ __forceinline__ void csr_rows(const int *__restrict__ ptr, const int *__restrict__ idx,
                                         const VT *__restrict__ val, const int *__restrict__ blk,
                                         int nblk, XF xload, PF pre_load, EPI epi, SpmvStage<VT, AT> *stages)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    SpmvStage<VT, AT> &st = stages[w];
    const int nwarps = gridDim.x * SPMV_WARPS;
    int b = blockIdx.x * SPMV_WARPS + w;
    if (b >= nblk) return;
    int r0 = blk[b], r1 = blk[b + 1];
    int e0 = ptr[r0], e1 = ptr[r1];
    while (true) {
        const int nr = r1 - r0;
        const int bn = b + nwarps;
        // next block's bounds (first level), overlapped with this block
        int nr0 = 0, nr1 = 0;
        if (bn < nblk) { nr0 = blk[bn]; nr1 = blk[bn + 1]; }
        if (e1 - e0 <= NNZ_W) {
            int ci[SPMV_PER_LANE];
            VT vv[SPMV_PER_LANE];
            AT xv[SPMV_PER_LANE];
#pragma unroll
            for (int t = 0; t < SPMV_PER_LANE; t++) {
                const int e = e0 + lane + 32 * t;
                ci[t] = 0;
                vv[t] = 0;
                if (e < e1) { ci[t] = idx[e]; vv[t] = val[e]; }
            }
            const int myrow = r0 + lane;
            const int myptr = (lane <= nr) ? ptr[myrow] : 0;
            const double mypre = (lane < nr) ? pre_load(myrow) : 0.0;
#pragma unroll
            for (int t = 0; t < SPMV_PER_LANE; t++) {
                const int e = e0 + lane + 32 * t;
                xv[t] = (e < e1) ? (AT)xload(ci[t]) : (AT)0;
            }
            // next block's row pointers (second level)
            int ne0 = 0, ne1 = 0;
            if (bn < nblk) { ne0 = ptr[nr0]; ne1 = ptr[nr1]; }
#pragma unroll
            for (int t = 0; t < SPMV_PER_LANE; t++) {
                const int q = lane + 32 * t;
                st.val[q] = vv[t];
                st.xv[q] = xv[t];
            }
            __syncwarp();
            int g = 32;
            while (g > 1 && g * nr > 32) g >>= 1;
            const int k = lane / g, lig = lane % g;
            const int r = r0 + k;
            const int a = __shfl_sync(0xffffffffu, myptr, k) - e0;
            const int zn = __shfl_sync(0xffffffffu, myptr, (k + 1) & 31);
            // the last row of a 32-row block ends at e1 (there is no lane 32)
            const int z = ((k + 1 == nr) ? e1 : zn) - e0;
            const double pre = __shfl_sync(0xffffffffu, mypre, k);
            AT acc = 0;
            if (r < r1)
                for (int q = a + lig; q < z; q += g) acc = fma((AT)st.val[q], st.xv[q], acc);
            for (int o = g >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, g);
            if (r < r1 && lig == 0) epi(r, (double)acc, pre);
            __syncwarp();
            b = bn;
            if (b >= nblk) break;
            r0 = nr0; r1 = nr1; e0 = ne0; e1 = ne1;
        } else {
            // one long row, streamed by the whole warp
            const double pre = pre_load(r0);
            AT acc = 0;
            int e = e0 + lane;
            for (; e + 96 < e1; e += 128) {
                const int c0 = idx[e], c1 = idx[e + 32], c2 = idx[e + 64], c3 = idx[e + 96];
                const VT v0 = val[e], v1 = val[e + 32], v2 = val[e + 64], v3 = val[e + 96];
                const AT x0 = (AT)xload(c0), x1 = (AT)xload(c1), x2 = (AT)xload(c2), x3 = (AT)xload(c3);
                acc = fma((AT)v0, x0, acc);
                acc = fma((AT)v1, x1, acc);
                acc = fma((AT)v2, x2, acc);
                acc = fma((AT)v3, x3, acc);
            }
            for (; e < e1; e += 32) acc = fma((AT)val[e], (AT)xload(idx[e]), acc);
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) epi(r0, (double)acc, pre);
            b = bn;
            if (b >= nblk) break;
            r0 = nr0; r1 = nr1;
            e0 = ptr[r0]; e1 = ptr[r1];
        }
    }
}

}  // namespace pgb
