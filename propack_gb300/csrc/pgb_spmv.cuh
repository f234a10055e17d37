// pgb_spmv.cuh -- the CSR sparse matrix-vector cores shared by the plain
// operator application and the fused Lanczos steps.  Two row schedules,
// chosen per matrix when the operator is built (Csr::short_rows):
//
// staged (rows of ~16 and more nonzeros): row blocks of at most ROWS_W rows
//   and NNZ_W nonzeros, or one long row.  Each warp owns whole blocks and
//   works without CTA barriers: every lane issues all of its (index, value)
//   loads for the block, then all of its gathers x[index], and parks value
//   and gathered input in its warp's slice of shared memory.  g lanes per
//   row (g = 32 / rows in the block, a power of two) then form the row sums
//   from shared memory.  A long row is streamed by the whole warp.
//
// short (most rows shorter than ~16): a warp takes 32 consecutive rows, one
//   lane per row; each lane walks its row in order with four (index, value)
//   pairs and four gathers in flight, so an instruction per nonzero and
//   lane is all the row costs.  Rows longer than SHORT_MAX are skipped by
//   the tiles and streamed afterwards, a whole warp per row, from a list.
//
// Summation order depends only on the matrix, never on timing, so results
// are bit-reproducible.
#pragma once
#include "pgb.cuh"

namespace pgb {

constexpr int SPMV_WARPS = BS / 32;  // warps per CTA
constexpr int SHORT_MAX = 48;        // longest row a lane sums alone (short schedule)

// One warp's shared-memory stage of the staged schedule: the block's
// values and gathered inputs.
template <typename VT, typename AT>
struct SpmvStage {
    VT val[NNZ_W];
    AT xv[NNZ_W];
};

constexpr int SPMV_PER_LANE = NNZ_W / 32;  // staged nonzeros per lane

// Visit every row; epi(row, sum, pre) is called by exactly one lane per row,
// where pre = pre_load(row) was issued early (with the row's own loads) so
// that per-row epilogue inputs never add a round trip.  xload(col) returns
// the gathered input for a column.  AT is the accumulation type (double for
// the FP64 path, float for FP32).
template <typename VT, typename AT, typename XF, typename PF, typename EPI>
__device__ __forceinline__ void csr_rows_staged(const int *__restrict__ ptr, const int *__restrict__ idx,
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


// the short-row schedule (see the top of the file).  Rows longer than
// SHORT_MAX are skipped by the tiles and streamed afterwards, one whole warp
// per row, from the matrix's list of long rows; the bounds of a warp's next
// tile are loaded with the current tile's first pairs.
template <typename VT, typename AT, typename XF, typename PF, typename EPI>
__device__ __forceinline__ void csr_rows_short(const int *__restrict__ ptr, const int *__restrict__ idx,
                                               const VT *__restrict__ val, int nrows, const int *__restrict__ longrows,
                                               int nlong, XF xload, PF pre_load, EPI epi)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * SPMV_WARPS;
    const int gw = blockIdx.x * SPMV_WARPS + (threadIdx.x >> 5);
    const int ntiles = (nrows + 31) / 32;
    int tile = gw;
    if (tile < ntiles) {
        int r = tile * 32 + lane;
        int e0 = r < nrows ? ptr[r] : 0;
        int e1 = r < nrows ? ptr[r + 1] : 0;
        while (true) {
            const bool own = r < nrows && e1 - e0 <= SHORT_MAX;
            const double pre = own ? pre_load(r) : 0.0;
            const int ntile = tile + nwarps;
            const int rn = ntile * 32 + lane;
            int n0 = 0, n1 = 0;
            if (ntile < ntiles && rn < nrows) { n0 = ptr[rn]; n1 = ptr[rn + 1]; }
            if (own) {
                AT acc = 0;
                int e = e0;
                for (; e + 3 < e1; e += 4) {
                    const int c0 = idx[e], c1 = idx[e + 1], c2 = idx[e + 2], c3 = idx[e + 3];
                    const VT v0 = val[e], v1 = val[e + 1], v2 = val[e + 2], v3 = val[e + 3];
                    const AT x0 = (AT)xload(c0), x1 = (AT)xload(c1), x2 = (AT)xload(c2), x3 = (AT)xload(c3);
                    acc = fma((AT)v0, x0, acc);
                    acc = fma((AT)v1, x1, acc);
                    acc = fma((AT)v2, x2, acc);
                    acc = fma((AT)v3, x3, acc);
                }
                for (; e < e1; e++) acc = fma((AT)val[e], (AT)xload(idx[e]), acc);
                epi(r, (double)acc, pre);
            }
            tile = ntile;
            if (tile >= ntiles) break;
            r = rn;
            e0 = n0;
            e1 = n1;
        }
    }
    for (int li = gw; li < nlong; li += nwarps) {
        const int r = longrows[li];
        const int f0 = ptr[r], f1 = ptr[r + 1];
        const double pre = lane == 0 ? pre_load(r) : 0.0;
        AT s = 0;
        int e = f0 + lane;
        for (; e + 96 < f1; e += 128) {
            const int c0 = idx[e], c1 = idx[e + 32], c2 = idx[e + 64], c3 = idx[e + 96];
            const VT v0 = val[e], v1 = val[e + 32], v2 = val[e + 64], v3 = val[e + 96];
            const AT x0 = (AT)xload(c0), x1 = (AT)xload(c1), x2 = (AT)xload(c2), x3 = (AT)xload(c3);
            s = fma((AT)v0, x0, s);
            s = fma((AT)v1, x1, s);
            s = fma((AT)v2, x2, s);
            s = fma((AT)v3, x3, s);
        }
        for (; e < f1; e += 32) s = fma((AT)val[e], (AT)xload(idx[e]), s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        if (lane == 0) epi(r, (double)s, pre);
    }
}

// the schedule chosen for the matrix
template <typename VT, typename AT, typename XF, typename PF, typename EPI>
__device__ __forceinline__ void csr_spmv(const Csr &A, const VT *__restrict__ val, XF xload, PF pre_load, EPI epi,
                                         SpmvStage<VT, AT> *stages)
{
    if (A.short_rows) csr_rows_short<VT, AT>(A.ptr, A.idx, val, A.rows, A.longrows, A.nlong, xload, pre_load, epi);
    else csr_rows_staged<VT, AT>(A.ptr, A.idx, val, A.blk, A.nblk, xload, pre_load, epi, stages);
}

}  // namespace pgb
