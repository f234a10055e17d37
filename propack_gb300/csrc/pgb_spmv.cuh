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
// chunked (rows shorter than ~16 on average): a warp takes 32 consecutive
//   rows (a tile; each warp a contiguous range of tiles holding an equal
//   share of the entries) and splits the tile's E entries, in CSR order, into 32
//   runs of C = ceil(E / 32) entries, one run per lane, whatever the row
//   lengths.  The operator build stores the tile's entries run-interleaved
//   (entry p at unit p % C, lane p / C), so every (index, value) load of
//   the warp is one coalesced 128/256-byte access, and every lane issues
//   the same C FP64 FMAs: a tile's FMA count is E / 32 instead of the
//   length of its longest row, which matters on a GPU whose FP64 pipe
//   retires two lanes per clock.  A row that ends inside a run is summed
//   by that lane alone, in CSR order; a row spread over several runs adds
//   the runs' partial sums in lane order.
//
// Summation order depends only on the matrix, never on timing, so results
// are bit-reproducible.
#pragma once
#include <climits>

#include "pgb.cuh"

namespace pgb {

constexpr int SPMV_WARPS = BS / 32;  // warps per CTA
constexpr int CHUNK_UNROLL = 4;      // chunked schedule: (index, value) pairs and gathers in flight per lane
constexpr int CHUNK_TILE_COST = 4;   // chunked schedule: fixed cost of a tile, in units of 32 entries

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


template <typename VT>
__device__ __forceinline__ const VT *chunk_vals(const Csr &A);
template <>
__device__ __forceinline__ const double *chunk_vals<double>(const Csr &A) { return A.cval; }
template <>
__device__ __forceinline__ const float *chunk_vals<float>(const Csr &A) { return A.cvalf; }
template <>
__device__ __forceinline__ const double2 *chunk_vals<double2>(const Csr &A) { return A.czval; }

// The chunked schedule's arithmetic on its accumulation type: real (float,
// double) or complex (double2 = (re, im); a complex entry costs four FP64
// FMAs on one index and one 16-byte gather, where the 2x2-block real form
// reads four entries)
template <typename AT>
__device__ __forceinline__ AT spmv_zero() { return (AT)0; }
template <>
__device__ __forceinline__ double2 spmv_zero<double2>() { return make_double2(0.0, 0.0); }
__device__ __forceinline__ float spmv_mac(float v, float x, float acc) { return fmaf(v, x, acc); }
__device__ __forceinline__ double spmv_mac(double v, double x, double acc) { return fma(v, x, acc); }
__device__ __forceinline__ double2 spmv_mac(double2 v, double2 x, double2 acc)
{
    acc.x = fma(v.x, x.x, acc.x);
    acc.x = fma(-v.y, x.y, acc.x);
    acc.y = fma(v.x, x.y, acc.y);
    acc.y = fma(v.y, x.x, acc.y);
    return acc;
}
__device__ __forceinline__ float spmv_add(float a, float b) { return a + b; }
__device__ __forceinline__ double spmv_add(double a, double b) { return a + b; }
__device__ __forceinline__ double2 spmv_add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }

template <typename AT>
struct ChunkStage {
    AT part[32];  // row q: the sum of its entries in the run where it ends
    AT tail[32];  // lane l: the sum of the row still open at the end of its run
    int bnd[33];  // row bounds of the tile, relative to its first entry
};

// warp_lower_bound2: for two keys, the first i in [0, n) with
// t[i] + kappa i >= key (non-decreasing in i, and >= key at n-1), each by a
// 32-way search of the whole warp.
// The two searches run in lockstep: each round issues both probes' loads
// before either ballot, so the pair costs the round trips of one search.
__device__ __forceinline__ void warp_lower_bound2(const int *__restrict__ t, int n, long long key0, long long key1,
                                                  int kappa, int &r0, int &r1)
{
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    auto ge = [&](int i, int v, long long key) { return (long long)v + (long long)kappa * i >= key; };
    auto narrow = [&](int &lo, int &hi, int step, unsigned m) {
        if (m == 0) {
            lo = min(lo + 31 * step + 1, hi);
        } else {
            const int f = __ffs(m) - 1;
            const int nhi = min(lo + f * step, hi);
            lo = f > 0 ? lo + (f - 1) * step + 1 : lo;
            hi = nhi;
        }
    };
    int lo0 = 0, hi0 = n, lo1 = 0, hi1 = n;
    while (hi0 - lo0 > 32 || hi1 - lo1 > 32) {
        const bool a0 = hi0 - lo0 > 32, a1 = hi1 - lo1 > 32;  // warp-uniform
        const int st0 = (hi0 - lo0 + 31) / 32, st1 = (hi1 - lo1 + 31) / 32;
        const int i0 = min(lo0 + lane * st0, hi0 - 1), i1 = min(lo1 + lane * st1, hi1 - 1);
        const int v0 = a0 ? t[i0] : 0, v1 = a1 ? t[i1] : 0;
        const unsigned m0 = __ballot_sync(FULL, a0 && ge(i0, v0, key0));
        const unsigned m1 = __ballot_sync(FULL, a1 && ge(i1, v1, key1));
        if (a0) narrow(lo0, hi0, st0, m0);
        if (a1) narrow(lo1, hi1, st1, m1);
    }
    // a window of exactly 32 may hold its answer at hi (no lane probes it)
    const bool in0 = lo0 + lane < hi0, in1 = lo1 + lane < hi1;
    const int v0 = in0 ? t[lo0 + lane] : 0, v1 = in1 ? t[lo1 + lane] : 0;
    const unsigned m0 = __ballot_sync(FULL, in0 ? ge(lo0 + lane, v0, key0) : true);
    const unsigned m1 = __ballot_sync(FULL, in1 ? ge(lo1 + lane, v1, key1) : true);
    r0 = m0 ? lo0 + __ffs(m0) - 1 : hi0;
    r1 = m1 ? lo1 + __ffs(m1) - 1 : hi1;
}

// the chunked schedule's tiles of this warp: a contiguous range holding an
// equal share of the work, counted as the tiles' units plus
// CHUNK_TILE_COST per tile (bounds, combine, epilogue), so that no warp of
// a CTA waits long for the others at the closing reductions.  Kernels call
// it before their first dependent load, so that its round trips overlap
// those of their control words.
__device__ __forceinline__ void chunk_warp_tiles(const int *__restrict__ tbase, int nrows, int &tb0, int &tb1)
{
    const int nwarps = gridDim.x * SPMV_WARPS;
    const int ntiles = (nrows + 31) / 32;
    const long long gw = blockIdx.x * SPMV_WARPS + (threadIdx.x >> 5);
    const long long work = (long long)tbase[ntiles] + (long long)CHUNK_TILE_COST * ntiles;
    warp_lower_bound2(tbase, ntiles + 1, work * gw / nwarps, work * (gw + 1) / nwarps, CHUNK_TILE_COST, tb0, tb1);
}

// tb0 < 0: the warp's tiles are found here (chunk_warp_tiles)
template <typename VT, typename AT, int UNROLL = CHUNK_UNROLL, typename XF, typename PF, typename EPI>
__device__ __forceinline__ void csr_rows_chunked(const int *__restrict__ ptr, const int *__restrict__ tbase,
                                                 const int *__restrict__ cidx, const VT *__restrict__ cval,
                                                 int nrows, XF xload, PF pre_load, EPI epi, ChunkStage<AT> *stages,
                                                 int tb0 = -1, int tb1 = -1)
{
    const int lane = threadIdx.x & 31;
    ChunkStage<AT> &cs = stages[threadIdx.x >> 5];
    if (tb0 < 0) chunk_warp_tiles(tbase, nrows, tb0, tb1);
    // a tile's bounds: lane l's row start (rows past the end are empty),
    // lane 31 also the tile's end, and the tile's units; those of the next
    // tile are loaded while the current one runs
    int lo_c = 0, end_c = 0, t0_c = 0, t1_c = 0;
    auto fetch = [&](int tile, int &lo_raw, int &end31, int &u0, int &u1) {
        const int rr = tile * 32 + lane;
        lo_raw = ptr[min(rr, nrows)];
        end31 = lane == 31 ? ptr[min(rr + 1, nrows)] : 0;
        u0 = tbase[tile];
        u1 = tbase[tile + 1];
    };
    if (tb0 < tb1) fetch(tb0, lo_c, end_c, t0_c, t1_c);
    for (int tile = tb0; tile < tb1; tile++) {
        const int r = tile * 32 + lane;
        int lo_n = 0, end_n = 0, t0_n = 0, t1_n = 0;
        if (tile + 1 < tb1) fetch(tile + 1, lo_n, end_n, t0_n, t1_n);
        const int eb = __shfl_sync(0xffffffffu, lo_c, 0);
        const int hi_raw = __shfl_down_sync(0xffffffffu, lo_c, 1);
        const int lo = lo_c - eb;
        const int hi = (lane == 31 ? end_c : hi_raw) - eb;
        const int t0 = t0_c, C = t1_c - t0_c;  // C >= 1
        lo_c = lo_n;
        end_c = end_n;
        t0_c = t0_n;
        t1_c = t1_n;
        using PT = decltype(pre_load(0));
        const PT pre = r < nrows ? pre_load(r) : PT{};
        cs.bnd[lane] = lo;
        if (lane == 31) cs.bnd[32] = hi;
        cs.part[lane] = spmv_zero<AT>();
        __syncwarp();
        // the row holding the run's first entry p0: the last q with
        // bnd[q] <= p0 (a non-empty row), or 32 when p0 is past the entries
        const int p0 = lane * C;
        int q = 0;
#pragma unroll
        for (int st = 16; st > 0; st >>= 1)
            if (cs.bnd[q + st] <= p0) q += st;
        if (cs.bnd[32] <= p0) q = 32;
        int nend = q < 32 ? cs.bnd[q + 1] : INT_MAX;
        int p = p0;
        AT acc = spmv_zero<AT>();
        const size_t off = (size_t)t0 * 32 + lane;
        const int *ci = cidx + off;
        const VT *cv = cval + off;
        // one entry of the run; closes row q when it ends at this entry
        auto step = [&](VT v, AT xv) {
            acc = spmv_mac((AT)v, xv, acc);
            if (++p == nend) {
                cs.part[q] = acc;
                acc = spmv_zero<AT>();
                do { ++q; } while (q < 32 && cs.bnd[q + 1] == p);
                nend = q < 32 ? cs.bnd[q + 1] : INT_MAX;
            }
        };
        int i = 0;
        for (; i + UNROLL - 1 < C; i += UNROLL) {
            int c[UNROLL];
            VT v[UNROLL];
            AT xv[UNROLL];
#pragma unroll
            for (int u = 0; u < UNROLL; u++) { c[u] = ci[32 * (i + u)]; v[u] = cv[32 * (i + u)]; }
#pragma unroll
            for (int u = 0; u < UNROLL; u++) xv[u] = (AT)xload(c[u]);
#pragma unroll
            for (int u = 0; u < UNROLL; u++) step(v[u], xv[u]);
        }
        for (; i < C; i++) step(cv[32 * i], (AT)xload(ci[32 * i]));
        cs.tail[lane] = acc;
        __syncwarp();
        // row `lane`: its runs ls .. le, added in lane order
        AT tot = spmv_zero<AT>();
        if (lo < hi) {
            const int ls = lo / C, le = (hi - 1) / C;
            if (ls == le) {
                tot = cs.part[lane];
            } else {
                tot = cs.tail[ls];
                for (int l2 = ls + 1; l2 < le; l2++) tot = spmv_add(tot, cs.tail[l2]);
                tot = spmv_add(tot, cs.part[lane]);
            }
        }
        if (r < nrows) epi(r, tot, pre);
        __syncwarp();
    }
}

// the schedule chosen for the matrix
template <typename VT, typename AT, typename XF, typename PF, typename EPI>
__device__ __forceinline__ void csr_spmv(const Csr &A, const VT *__restrict__ val, XF xload, PF pre_load, EPI epi,
                                         SpmvStage<VT, AT> *stages, ChunkStage<AT> *cstages)
{
    if (A.short_rows)
        csr_rows_chunked<VT, AT>(A.ptr, A.tbase, A.cidx, chunk_vals<VT>(A), A.rows, xload, pre_load, epi, cstages);
    else csr_rows_staged<VT, AT>(A.ptr, A.idx, val, A.blk, A.nblk, xload, pre_load, epi, stages);
}

}  // namespace pgb
