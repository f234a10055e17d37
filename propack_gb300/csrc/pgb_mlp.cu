// pgb_mlp.cu -- the learned start vector: a row-wise MLP that stands in for
// dgetu0's random start (double/dgetu0.F:11-89) on families of related
// matrices.  No reference counterpart; the random start stays the fallback.
//
// Per row i of A the network reads MLP_IN features
//   f0 = log1p(nnz of row i) / 4,
//   f1 = ||y_i|| / rho,  f2..f17 = 2 y_i / rho,
// where y = A Omega is a 16-column Gaussian sketch (Omega from a counter-based
// generator, so the sketch is reproducible) and rho the RMS of ||y_i||; it
// outputs one entry of the start vector u0:
//   h1 = relu(W1 f + b1), h2 = relu(W2 h1 + b2), u0_i = w3 . h2 + b3
// (18 -> 256 -> 256 -> 1).  Weights are held in FP32 (Adam master copy) and
// used as BF16; every product accumulates in FP32.  The 256 x 256 layer runs
// on the 5th-generation tensor cores (tcgen05.mma, FP32 accumulators in
// tensor memory), forward and backward through its input; the mma.sync
// kernel it replaced stays selectable (propack_mlp_set_impl) as the
// reference implementation.
//
// Training (propack_mlp_train_step) minimises, for a matrix whose leading k
// left singular vectors U are known,
//   L(u0) = -(1/k) sum_j log(c_j^2 + eps ||u0||^2 / k) + log ||u0||^2,
//   c = U' u0,
// which is small when u0 lies in span(U) with every c_j of similar size, the
// property that makes every wanted Ritz value converge early.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <map>
#include <vector>

#include <atomic>

#include "../../include/propack_gb300.h"
#include "pgb.cuh"
#include "pgb_tc.cuh"

namespace pgb {

constexpr int MLP_IN = 18, MLP_H = 256, MLP_SK = 16;
constexpr int OW1 = 0, OB1 = OW1 + MLP_H * MLP_IN, OW2 = OB1 + MLP_H, OB2 = OW2 + MLP_H * MLP_H,
              OW3 = OB2 + MLP_H, OB3 = OW3 + MLP_H, MLP_NP = OB3 + 1;
constexpr int W2S = MLP_H + 8;  // padded row stride of the BF16 W2 copies in shared memory
constexpr double MLP_EPS = 1e-4;

typedef __nv_bfloat16 bf16;

struct Mlp {
    float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;  // MLP_NP each
    bf16 *W1b = nullptr, *W2b = nullptr, *W2Tb = nullptr, *w3b = nullptr;
    int64_t step = 0;
    int cap = 0;
    int64_t ucap = 0;
    float *F = nullptr, *out = nullptr, *gout = nullptr, *D1 = nullptr;
    bf16 *H1 = nullptr, *H2 = nullptr, *D2 = nullptr;
    double *Y = nullptr, *om = nullptr, *U = nullptr, *red = nullptr, *coef = nullptr;
    float *part = nullptr;  // per-CTA partial sums of the reductions
    int *err = nullptr;     // set by the tensor-core kernel when a bounded wait runs out
    int device = 0;
    cudaStream_t s = nullptr;
};

// ------------------------------------------------------------- helpers
__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// Omega(j, c): standard normal from two counter-based uniforms (Box-Muller)
__global__ void k_mlp_omega(int n, int col, unsigned long long seed, double *x)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const unsigned long long a = mix64(seed ^ mix64(((unsigned long long)col << 40) ^ (unsigned long long)j));
        const unsigned long long b = mix64(a);
        const double u1 = ((double)(a >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        const double u2 = (double)(b >> 11) * (1.0 / 9007199254740992.0);
        x[j] = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
    }
}

// sum over rows of ||y_i||^2 (Y column-major m x 16): partials per CTA
__global__ void __launch_bounds__(256) k_mlp_sumsq(int m, const double *Y, double *part)
{
    __shared__ double red[32];
    double s = 0.0;
    for (int i = blockIdx.x * 256 + threadIdx.x; i < m; i += gridDim.x * 256)
        for (int c = 0; c < MLP_SK; c++) {
            const double y = Y[(size_t)c * m + i];
            s = fma(y, y, s);
        }
    s = block_sum<256>(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_mlp_features(int m, const int *rowptr, const double *Y, const double *part, int nparts, float *F)
{
    __shared__ double rho;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < nparts; b++) s += part[b];
        rho = sqrt(s / (double)m);
        if (!(rho > 0.0)) rho = 1.0;
    }
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        float *f = F + (size_t)i * MLP_IN;
        double nn = 0.0;
        for (int c = 0; c < MLP_SK; c++) {
            const double y = Y[(size_t)c * m + i] / rho;
            nn = fma(y, y, nn);
            f[2 + c] = (float)(2.0 * y);
        }
        f[0] = (float)(log1p((double)(rowptr[i + 1] - rowptr[i])) / 4.0);
        f[1] = (float)sqrt(nn);
    }
}

// h1 = relu(W1 f + b1) as BF16, row-major m x 256; one thread per (row, unit)
__global__ void __launch_bounds__(MLP_H) k_mlp_l1(int m, const float *F, const bf16 *W1b, const float *b1, bf16 *H1)
{
    __shared__ float w[MLP_H * MLP_IN];
    for (int t = threadIdx.x; t < MLP_H * MLP_IN; t += MLP_H) w[t] = __bfloat162float(W1b[t]);
    __syncthreads();
    const int j = threadIdx.x;
    const float bj = b1[j];
    for (int i = blockIdx.x; i < m; i += gridDim.x) {
        const float *f = F + (size_t)i * MLP_IN;
        float z = bj;
#pragma unroll
        for (int q = 0; q < MLP_IN; q++) z = fmaf(w[j * MLP_IN + q], f[q], z);
        H1[(size_t)i * MLP_H + j] = __float2bfloat16_rn(fmaxf(z, 0.f));
    }
}

__device__ __forceinline__ void mma16816(float c[4], const unsigned a[4], unsigned b0, unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Z = X Wt' (X: m x 256 BF16 row-major; Wt: 256 x 256 BF16 [n][k]) on the
// tensor cores, one warp per 16 rows and all 256 columns.  MODE 0 (forward
// layer 2): out = bf16(relu(Z + bias)) -> Ob.  MODE 1 (backward through
// layer 2): out = Z * (mask > 0) -> Of (FP32), mask = H1.
template <int MODE>
__global__ void __launch_bounds__(256) k_mlp_mm(int m, const bf16 *X, const bf16 *Wt, const float *bias,
                                               const bf16 *mask, bf16 *Ob, float *Of)
{
    extern __shared__ unsigned short wsm[];  // 256 x W2S
    for (int t = threadIdx.x; t < MLP_H * MLP_H / 2; t += blockDim.x) {
        const int n = t / (MLP_H / 2), k2 = t % (MLP_H / 2);
        reinterpret_cast<unsigned *>(wsm)[(n * W2S) / 2 + k2] = reinterpret_cast<const unsigned *>(Wt)[t];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, gid = lane >> 2, tig = lane & 3;
    const int nw = blockDim.x / 32;
    for (int r0 = (blockIdx.x * nw + (threadIdx.x >> 5)) * 16; r0 < m; r0 += gridDim.x * nw * 16) {
        const int ra = r0 + gid, rb = ra + 8;
        float acc[32][4];
#pragma unroll
        for (int t = 0; t < 32; t++) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
        for (int k0 = 0; k0 < MLP_H; k0 += 16) {
            unsigned a[4];
            const unsigned *xa = reinterpret_cast<const unsigned *>(X + (size_t)ra * MLP_H + k0 + 2 * tig);
            const unsigned *xb = reinterpret_cast<const unsigned *>(X + (size_t)rb * MLP_H + k0 + 2 * tig);
            a[0] = ra < m ? xa[0] : 0u;
            a[1] = rb < m ? xb[0] : 0u;
            a[2] = ra < m ? xa[4] : 0u;
            a[3] = rb < m ? xb[4] : 0u;
#pragma unroll
            for (int t = 0; t < 32; t++) {
                const unsigned short *bp = wsm + (8 * t + gid) * W2S + k0 + 2 * tig;
                mma16816(acc[t], a, *reinterpret_cast<const unsigned *>(bp), *reinterpret_cast<const unsigned *>(bp + 8));
            }
        }
#pragma unroll
        for (int t = 0; t < 32; t++)
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int r = h ? rb : ra;
                if (r >= m) continue;
                const int c = 8 * t + 2 * tig;
                float z0 = acc[t][2 * h], z1 = acc[t][2 * h + 1];
                if (MODE == 0) {
                    z0 = fmaxf(z0 + bias[c], 0.f);
                    z1 = fmaxf(z1 + bias[c + 1], 0.f);
                    __nv_bfloat162 v;
                    v.x = __float2bfloat16_rn(z0);
                    v.y = __float2bfloat16_rn(z1);
                    *reinterpret_cast<__nv_bfloat162 *>(Ob + (size_t)r * MLP_H + c) = v;
                } else {
                    const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162 *>(mask + (size_t)r * MLP_H + c);
                    Of[(size_t)r * MLP_H + c] = __bfloat162float(mk.x) > 0.f ? z0 : 0.f;
                    Of[(size_t)r * MLP_H + c + 1] = __bfloat162float(mk.y) > 0.f ? z1 : 0.f;
                }
            }
    }
}

// The same product on the 5th-generation tensor cores.  A persistent CTA
// (256 threads, one per SM: 192 KB of shared memory) keeps Wt in shared
// memory in the no-swizzle K-major layout of pgb_tc.cuh (16 K steps of 256
// rows x 16 K) and takes tiles of 128 rows of X in turn: the threads write
// the tile into the same layout (two lanes per 32-byte sector of a row, so
// that the loads are whole sectors and a warp's stores take the minimum
// four wavefronts), thread 0 issues the 16 MMAs (M = 128, N = 256, K = 16,
// BF16 x BF16 -> FP32) into TMEM columns 0..255 and commits them to an
// mbarrier, and every warp reads 32 TMEM lanes (rows; lanes 32 (w mod 4)..)
// x 128 columns (half w / 4) with tcgen05.ld and applies k_mlp_mm's
// epilogue.  Every wait is bounded; one that runs out sets *err and the CTA
// stops after its MMAs in flight are done.
constexpr int TM_BM = 128, TM_N = MLP_H, TM_KSTEPS = MLP_H / 16;
constexpr int TM_ATILE = TM_BM * 16 * 2;  // 4096 bytes per K step
constexpr int TM_BTILE = TM_N * 16 * 2;   // 8192 bytes per K step
constexpr int TM_SMEM = TM_KSTEPS * (TM_ATILE + TM_BTILE) + 128;
constexpr uint32_t TM_IDESC = tc_idesc_bf16(TM_BM, TM_N);
constexpr unsigned TM_TMEM_COLS = TM_N;
constexpr long TM_WAIT_LIMIT = 1L << 22;
static_assert(TM_SMEM <= 227 * 1024, "shared memory");

template <int MODE>
__global__ void __launch_bounds__(256, 1) k_mlp_mm_tc(int m, const bf16 *X, const bf16 *Wt, const float *bias,
                                                      const bf16 *mask, bf16 *Ob, float *Of, int *err)
{
    extern __shared__ __align__(1024) unsigned char tm_sm[];
    const uint32_t a_s = tc_smem(tm_sm), b_s = a_s + TM_KSTEPS * TM_ATILE;
    uint64_t *bar = reinterpret_cast<uint64_t *>(tm_sm + TM_KSTEPS * (TM_ATILE + TM_BTILE));
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
    int *sbad = reinterpret_cast<int *>(tslot + 1);
    const uint32_t bar_s = tc_smem(bar);
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int ntiles = (m + TM_BM - 1) / TM_BM;
    if (tid == 0) {
        tc_bar_init(bar_s, 1);
        *sbad = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(tslot)),
                     "r"(TM_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // Wt (256 rows n x 256 K) into shared memory, once per CTA
    for (int q = tid; q < TM_N * (MLP_H / 8); q += blockDim.x) {
        const int n = (q >> 1) & (TM_N - 1), kc = ((q >> 9) << 1) | (q & 1);
        const uint4 v = *reinterpret_cast<const uint4 *>(Wt + (size_t)n * MLP_H + kc * 8);
        tc_st16(b_s + (kc >> 1) * TM_BTILE + (n >> 3) * 256 + (kc & 1) * 128 + (n & 7) * 16, v);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    int it = 0;
    bool bad = false;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
        const int row0 = t * TM_BM;
        // the tile of X (rows past m read as zeros)
        for (int q = tid; q < TM_BM * (MLP_H / 8); q += blockDim.x) {
            const int r = (q >> 1) & (TM_BM - 1), kc = ((q >> 8) << 1) | (q & 1);
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (row0 + r < m) v = *reinterpret_cast<const uint4 *>(X + (size_t)(row0 + r) * MLP_H + kc * 8);
            tc_st16(a_s + (kc >> 1) * TM_ATILE + (r >> 3) * 256 + (kc & 1) * 128 + (r & 7) * 16, v);
        }
        tc_fence_proxy();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int ks = 0; ks < TM_KSTEPS; ks++)
                tc_mma(tmem, tc_desc(a_s + ks * TM_ATILE), tc_desc(b_s + ks * TM_BTILE), TM_IDESC, ks > 0 ? 1u : 0u);
            tc_commit(bar_s);
        }
        const bool ok = tc_bar_wait(bar_s, (unsigned)(it & 1), TM_WAIT_LIMIT);
        if (__syncthreads_or(!ok)) {
            bad = true;
            break;
        }
        tc_fence_after();
        {
            const int L = 32 * (w & 3), cb = (w >> 2) * (TM_N / 2);
            const int row = row0 + L + lane;
#pragma unroll 1
            for (int cc = 0; cc < TM_N / 2; cc += 8) {
                uint32_t v[8];
                tc_ld8(tmem + ((uint32_t)L << 16) + (uint32_t)(cb + cc), v);
                tc_wait_ld();
                if (row >= m) continue;
                const int c = cb + cc;
                if (MODE == 0) {
                    uint32_t pk[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const float z0 = fmaxf(__uint_as_float(v[2 * j]) + bias[c + 2 * j], 0.f);
                        const float z1 = fmaxf(__uint_as_float(v[2 * j + 1]) + bias[c + 2 * j + 1], 0.f);
                        __nv_bfloat162 h;
                        h.x = __float2bfloat16_rn(z0);
                        h.y = __float2bfloat16_rn(z1);
                        pk[j] = *reinterpret_cast<uint32_t *>(&h);
                    }
                    *reinterpret_cast<uint4 *>(Ob + (size_t)row * MLP_H + c) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                } else {
                    const uint4 mk = *reinterpret_cast<const uint4 *>(mask + (size_t)row * MLP_H + c);
                    const uint32_t mw[4] = {mk.x, mk.y, mk.z, mk.w};
                    float o[8];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162 *>(&mw[j]);
                        o[2 * j] = __bfloat162float(h.x) > 0.f ? __uint_as_float(v[2 * j]) : 0.f;
                        o[2 * j + 1] = __bfloat162float(h.y) > 0.f ? __uint_as_float(v[2 * j + 1]) : 0.f;
                    }
                    float4 *dst = reinterpret_cast<float4 *>(Of + (size_t)row * MLP_H + c);
                    dst[0] = make_float4(o[0], o[1], o[2], o[3]);
                    dst[1] = make_float4(o[4], o[5], o[6], o[7]);
                }
            }
        }
        // the TMEM reads are done before the next tile's MMAs overwrite the
        // accumulators, and the MMAs before the next tile's X overwrites A
        tc_fence_before();
        __syncthreads();
    }
    if (bad) {
        if (tid == 0) atomicExch(err, 1);
        tc_bar_wait(bar_s, (unsigned)(it & 1), TM_WAIT_LIMIT);  // the MMAs in flight (bounded)
    }
    tc_fence_before();
    __syncthreads();
    if (w == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TM_TMEM_COLS) : "memory");
}

// u0_i = w3 . h2_i + b3, one warp per row
__global__ void k_mlp_l3(int m, const bf16 *H2, const bf16 *w3b, const float *b3, float *out)
{
    const int lane = threadIdx.x & 31;
    for (int i = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); i < m; i += gridDim.x * (blockDim.x / 32)) {
        float s = 0.f;
        for (int j = lane; j < MLP_H; j += 32) s = fmaf(__bfloat162float(w3b[j]), __bfloat162float(H2[(size_t)i * MLP_H + j]), s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[i] = s + b3[0];
    }
}

// partials of c = U' u0 (k values) and ||u0||^2: part[b * (k+1) + j]
__global__ void __launch_bounds__(256) k_mlp_proj(int m, int k, const double *U, const float *out, double *part)
{
    __shared__ double red[32];
    for (int j = 0; j <= k; j++) {
        double s = 0.0;
        for (int i = blockIdx.x * 256 + threadIdx.x; i < m; i += gridDim.x * 256) {
            const double o = out[i];
            s = fma(j < k ? U[(size_t)j * m + i] : o, o, s);
        }
        s = block_sum<256>(s, red);
        if (threadIdx.x == 0) part[(size_t)blockIdx.x * (k + 1) + j] = s;
    }
}

// dL/du0_i = sum_j U_ij coef_j + coef_k u0_i
__global__ void k_mlp_gout(int m, int k, const double *U, const double *coef, const float *out, float *g)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        double s = coef[k] * (double)out[i];
        for (int j = 0; j < k; j++) s = fma(U[(size_t)j * m + i], coef[j], s);
        g[i] = (float)s;
    }
}

// layer 3 backward: partials of dw3 (256) and db3, and D2 = bf16(g w3 [h2 > 0])
__global__ void __launch_bounds__(MLP_H) k_mlp_b3(int m, const float *g, const bf16 *H2, const bf16 *w3b, bf16 *D2,
                                                  float *part)
{
    const int j = threadIdx.x;
    const float w = __bfloat162float(w3b[j]);
    float dw = 0.f, db = 0.f;
    for (int i = blockIdx.x; i < m; i += gridDim.x) {
        const float gi = g[i];
        const float h = __bfloat162float(H2[(size_t)i * MLP_H + j]);
        dw = fmaf(gi, h, dw);
        db += gi;
        D2[(size_t)i * MLP_H + j] = __float2bfloat16_rn(h > 0.f ? gi * w : 0.f);
    }
    part[(size_t)blockIdx.x * (MLP_H + 1) + j] = dw;
    if (j == 0) part[(size_t)blockIdx.x * (MLP_H + 1) + MLP_H] = db;
}

// dW2 = D2' H1 (256 x 256, summed over rows) and db2 = sum D2: CTA (tile,
// chunk) owns a 64 x 64 block of dW2 over one row chunk; partials per chunk
constexpr int DW_TR = 32;
__global__ void __launch_bounds__(256) k_mlp_dw2(int m, int chunk, const bf16 *D2, const bf16 *H1, float *part)
{
    __shared__ float dt[DW_TR][64 + 1], ht[DW_TR][64 + 1];
    const int tj = blockIdx.x / 4, tl = blockIdx.x % 4;  // 64-row block of j (D2 col), of l (H1 col)
    const int i0 = blockIdx.y * chunk, i1 = min(m, i0 + chunk);
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    float acc[4][4] = {};
    float dbs = 0.f;
    for (int ib = i0; ib < i1; ib += DW_TR) {
        for (int t = threadIdx.x; t < DW_TR * 64; t += 256) {
            const int r = t / 64, c = t % 64, i = ib + r;
            dt[r][c] = i < i1 ? __bfloat162float(D2[(size_t)i * MLP_H + tj * 64 + c]) : 0.f;
            ht[r][c] = i < i1 ? __bfloat162float(H1[(size_t)i * MLP_H + tl * 64 + c]) : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int r = 0; r < DW_TR; r++) {
            float dv[4], hv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) { dv[q] = dt[r][ty + 16 * q]; hv[q] = ht[r][tx + 16 * q]; }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[p][q] = fmaf(dv[p], hv[q], acc[p][q]);
        }
        if (tl == 0 && threadIdx.x < 64)
            for (int r = 0; r < DW_TR; r++) dbs += dt[r][threadIdx.x];
        __syncthreads();
    }
    float *P = part + (size_t)blockIdx.y * (MLP_H * MLP_H + MLP_H);
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++) P[(size_t)(tj * 64 + ty + 16 * p) * MLP_H + tl * 64 + tx + 16 * q] = acc[p][q];
    if (tl == 0 && threadIdx.x < 64) P[MLP_H * MLP_H + tj * 64 + threadIdx.x] = dbs;
}

// dW1 = D1' F (256 x 18) and db1 = sum D1: partials per CTA, thread = unit
__global__ void __launch_bounds__(MLP_H) k_mlp_dw1(int m, const float *D1, const float *F, float *part)
{
    const int j = threadIdx.x;
    float acc[MLP_IN + 1] = {};
    for (int i = blockIdx.x; i < m; i += gridDim.x) {
        const float d = D1[(size_t)i * MLP_H + j];
        const float *f = F + (size_t)i * MLP_IN;
#pragma unroll
        for (int q = 0; q < MLP_IN; q++) acc[q] = fmaf(d, f[q], acc[q]);
        acc[MLP_IN] += d;
    }
    float *P = part + (size_t)blockIdx.x * (MLP_H * (MLP_IN + 1));
#pragma unroll
    for (int q = 0; q <= MLP_IN; q++) P[(size_t)q * MLP_H + j] = acc[q];
}

// fixed-order sums of the partials into the flat gradient
__global__ void k_mlp_sum_b3(int nb, const float *part, float *g)
{
    const int j = threadIdx.x;  // 0..256
    if (j > MLP_H) return;
    float s = 0.f;
    for (int b = 0; b < nb; b++) s += part[(size_t)b * (MLP_H + 1) + j];
    if (j < MLP_H) g[OW3 + j] = s;
    else g[OB3] = s;
}
__global__ void k_mlp_sum_dw2(int nchunk, const float *part, float *g)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= MLP_H * MLP_H + MLP_H) return;
    float s = 0.f;
    for (int b = 0; b < nchunk; b++) s += part[(size_t)b * (MLP_H * MLP_H + MLP_H) + t];
    if (t < MLP_H * MLP_H) g[OW2 + t] = s;
    else g[OB2 + (t - MLP_H * MLP_H)] = s;
}
__global__ void k_mlp_sum_dw1(int nb, const float *part, float *g)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;  // q * 256 + j
    if (t >= MLP_H * (MLP_IN + 1)) return;
    float s = 0.f;
    for (int b = 0; b < nb; b++) s += part[(size_t)b * (MLP_H * (MLP_IN + 1)) + t];
    const int q = t / MLP_H, j = t % MLP_H;
    if (q < MLP_IN) g[OW1 + j * MLP_IN + q] = s;
    else g[OB1 + j] = s;
}

// Adam (Kingma & Ba 2015) on the FP32 master copy
__global__ void k_mlp_adam(float *p, const float *g, float *m1, float *m2, float lr, float c1, float c2)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= MLP_NP) return;
    const float gt = g[t];
    const float a = 0.9f * m1[t] + 0.1f * gt;
    const float b = 0.999f * m2[t] + 0.001f * gt * gt;
    m1[t] = a;
    m2[t] = b;
    p[t] -= lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
}

// BF16 compute copies of the weights (W2 also transposed)
__global__ void k_mlp_cast(const float *p, bf16 *W1b, bf16 *W2b, bf16 *W2Tb, bf16 *w3b)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < MLP_H * MLP_IN) W1b[t] = __float2bfloat16_rn(p[OW1 + t]);
    if (t < MLP_H * MLP_H) {
        const int n = t / MLP_H, k = t % MLP_H;
        const bf16 v = __float2bfloat16_rn(p[OW2 + t]);
        W2b[t] = v;                       // [out n][in k]
        W2Tb[(size_t)k * MLP_H + n] = v;  // [in k][out n]
    }
    if (t < MLP_H) w3b[t] = __float2bfloat16_rn(p[OW3 + t]);
}

// ------------------------------------------------------------ host side
static std::mutex g_mlp_mu;
static std::map<int64_t, Mlp *> g_mlps;
static int64_t g_mlp_next = 1;

static Mlp *lookup_mlp(int64_t h)
{
    std::lock_guard<std::mutex> lk(g_mlp_mu);
    auto it = g_mlps.find(h);
    return it == g_mlps.end() ? nullptr : it->second;
}

static void mlp_reserve(Mlp &M, int m, int k)
{
    if (m > M.cap) {
        for (void *q : {(void *)M.F, (void *)M.out, (void *)M.gout, (void *)M.D1, (void *)M.H1, (void *)M.H2,
                        (void *)M.D2, (void *)M.Y})
            if (q) cudaFree(q);
        PGB_CUDA(cudaMalloc(&M.F, sizeof(float) * (size_t)m * MLP_IN));
        PGB_CUDA(cudaMalloc(&M.out, sizeof(float) * (size_t)m));
        PGB_CUDA(cudaMalloc(&M.gout, sizeof(float) * (size_t)m));
        PGB_CUDA(cudaMalloc(&M.D1, sizeof(float) * (size_t)m * MLP_H));
        PGB_CUDA(cudaMalloc(&M.H1, sizeof(bf16) * (size_t)m * MLP_H));
        PGB_CUDA(cudaMalloc(&M.H2, sizeof(bf16) * (size_t)m * MLP_H));
        PGB_CUDA(cudaMalloc(&M.D2, sizeof(bf16) * (size_t)m * MLP_H));
        PGB_CUDA(cudaMalloc(&M.Y, sizeof(double) * (size_t)m * MLP_SK));
        M.cap = m;
    }
    const size_t need = (size_t)m * (size_t)std::max(k, 1);
    if (need > (size_t)M.ucap) {
        if (M.U) cudaFree(M.U);
        PGB_CUDA(cudaMalloc(&M.U, sizeof(double) * need));
        M.ucap = (int64_t)need;
    }
}

constexpr int MLP_GRID = 1024;         // CTAs of the row-parallel reductions
constexpr int MLP_DW2_CHUNKS = 64;     // row chunks of dW2

static void mlp_cast(Mlp &M)
{
    k_mlp_cast<<<(MLP_H * MLP_H + 255) / 256, 256, 0, M.s>>>(M.p, M.W1b, M.W2b, M.W2Tb, M.w3b);
    PGB_LAUNCHED();
}

// features of the operator's rows into M.F (m rows)
static void mlp_features(Mlp &M, const Operator &op, unsigned long long seed)
{
    const int m = op.m, n = op.n;
    mlp_reserve(M, m, 1);
    if (!M.om) PGB_CUDA(cudaMalloc(&M.om, sizeof(double) * (size_t)std::max(n, 1)));
    for (int c = 0; c < MLP_SK; c++) {
        k_mlp_omega<<<std::min(4096, (n + 255) / 256), 256, 0, M.s>>>(n, c, seed, M.om);
        PGB_LAUNCHED();
        op_apply<double>(op, false, M.om, M.Y + (size_t)c * m, M.s);
    }
    k_mlp_sumsq<<<MLP_GRID, 256, 0, M.s>>>(m, M.Y, M.red);
    PGB_LAUNCHED();
    k_mlp_features<<<std::min(4096, (m + 255) / 256), 256, 0, M.s>>>(m, op.fwd.ptr, M.Y, M.red, MLP_GRID, M.F);
    PGB_LAUNCHED();
}

static size_t mm_smem() { return sizeof(unsigned short) * MLP_H * W2S; }

// the 256 x 256 layer: 1 the tcgen05 kernel (default), 0 the mma.sync one
static std::atomic<int> g_mlp_impl{1};

// Z = X Wt' with the layer's epilogue (MODE 0 forward, 1 backward)
template <int MODE>
static void mlp_mm(Mlp &M, int m, const bf16 *X, const bf16 *Wt, const float *bias, const bf16 *mask, bf16 *Ob,
                   float *Of)
{
    if (g_mlp_impl.load() == 1) {
        const int g = std::max(1, std::min(device_info().sms, (m + TM_BM - 1) / TM_BM));
        k_mlp_mm_tc<MODE><<<g, 256, TM_SMEM, M.s>>>(m, X, Wt, bias, mask, Ob, Of, M.err);
    } else {
        const int g = std::min(device_info().sms, (m + 127) / 128);
        k_mlp_mm<MODE><<<g, 256, mm_smem(), M.s>>>(m, X, Wt, bias, mask, Ob, Of);
    }
    PGB_LAUNCHED();
}
// after the stream has been synchronised: a wait of the tensor-core kernel that ran out
static void mlp_check(Mlp &M)
{
    int e = 0;
    PGB_CUDA(cudaMemcpy(&e, M.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        PGB_CUDA(cudaMemset(M.err, 0, sizeof(int)));
        set_error("learned start: a tensor-core wait ran out");
        throw WaitFailure();
    }
}

static void mlp_forward(Mlp &M, int m)
{
    k_mlp_l1<<<std::min(8192, m), MLP_H, 0, M.s>>>(m, M.F, M.W1b, M.p + OB1, M.H1);
    PGB_LAUNCHED();
    mlp_mm<0>(M, m, M.H1, M.W2b, M.p + OB2, nullptr, M.H2, nullptr);
    k_mlp_l3<<<std::min(4096, (m + 7) / 8), 256, 0, M.s>>>(m, M.H2, M.w3b, M.p + OB3, M.out);
    PGB_LAUNCHED();
}

// loss and flat gradient for the matrix whose features sit in M.F and whose
// leading left singular vectors (m x k, column-major) sit in M.U
static double mlp_backward(Mlp &M, int m, int k)
{
    k_mlp_proj<<<MLP_GRID, 256, 0, M.s>>>(m, k, M.U, M.out, M.red);
    PGB_LAUNCHED();
    std::vector<double> part((size_t)MLP_GRID * (k + 1));
    PGB_CUDA(cudaMemcpyAsync(part.data(), M.red, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, M.s));
    PGB_CUDA(cudaStreamSynchronize(M.s));
    std::vector<double> c(k + 1, 0.0);
    for (int b = 0; b < MLP_GRID; b++)
        for (int j = 0; j <= k; j++) c[j] += part[(size_t)b * (k + 1) + j];
    const double nrm2 = std::max(c[k], 1e-300);
    const double eps = MLP_EPS * nrm2 / k;
    double loss = std::log(nrm2);
    std::vector<double> coef(k + 1);
    for (int j = 0; j < k; j++) {
        loss -= std::log(c[j] * c[j] + eps) / k;
        coef[j] = -2.0 * c[j] / ((c[j] * c[j] + eps) * k);
    }
    // d/du0 of log ||u0||^2 plus the eps ||u0||^2 terms
    double s = 0.0;
    for (int j = 0; j < k; j++) s += (MLP_EPS / k) / (c[j] * c[j] + eps);
    coef[k] = 2.0 / nrm2 - 2.0 * s / k;
    PGB_CUDA(cudaMemcpyAsync(M.coef, coef.data(), sizeof(double) * (k + 1), cudaMemcpyHostToDevice, M.s));
    k_mlp_gout<<<std::min(4096, (m + 255) / 256), 256, 0, M.s>>>(m, k, M.U, M.coef, M.out, M.gout);
    PGB_LAUNCHED();
    float *pf = reinterpret_cast<float *>(M.red);
    k_mlp_b3<<<MLP_GRID, MLP_H, 0, M.s>>>(m, M.gout, M.H2, M.w3b, M.D2, pf);
    PGB_LAUNCHED();
    k_mlp_sum_b3<<<1, 288, 0, M.s>>>(MLP_GRID, pf, M.g);
    PGB_LAUNCHED();
    const int chunk = (m + MLP_DW2_CHUNKS - 1) / MLP_DW2_CHUNKS;
    k_mlp_dw2<<<dim3(16, MLP_DW2_CHUNKS), 256, 0, M.s>>>(m, chunk, M.D2, M.H1, M.part);
    PGB_LAUNCHED();
    k_mlp_sum_dw2<<<(MLP_H * MLP_H + MLP_H + 255) / 256, 256, 0, M.s>>>(MLP_DW2_CHUNKS, M.part, M.g);
    PGB_LAUNCHED();
    mlp_mm<1>(M, m, M.D2, M.W2Tb, nullptr, M.H1, nullptr, M.D1);
    k_mlp_dw1<<<MLP_GRID, MLP_H, 0, M.s>>>(m, M.D1, M.F, pf);
    PGB_LAUNCHED();
    k_mlp_sum_dw1<<<(MLP_H * (MLP_IN + 1) + 255) / 256, 256, 0, M.s>>>(MLP_GRID, pf, M.g);
    PGB_LAUNCHED();
    return loss;
}

static Operator *mlp_operator(int64_t op_handle)
{
    Operator *op = lookup_operator(op_handle);
    if (!op) {
        set_error("no live operator handle");
        throw ArgFailure();
    }
    return op;
}

}  // namespace pgb

using namespace pgb;

#define MLP_TRY(...)                        \
    try {                                   \
        __VA_ARGS__;                        \
        return 0;                           \
    } catch (const ArgFailure &) {          \
        return PROPACK_ERR_ARG;             \
    } catch (const CudaFailure &) {         \
        return PROPACK_ERR_CUDA;            \
    } catch (const WaitFailure &) {         \
        return PROPACK_ERR_WAIT;            \
    }

extern "C" int propack_mlp_create(uint64_t seed, int64_t *handle)
{
    MLP_TRY({
        if (!handle) { set_error("propack_mlp_create: null handle"); throw ArgFailure(); }
        Mlp *M = new Mlp();
        PGB_CUDA(cudaGetDevice(&M->device));
        PGB_CUDA(cudaStreamCreateWithFlags(&M->s, cudaStreamNonBlocking));
        // He-style initialisation, drawn on the host (small)
        std::vector<float> p(MLP_NP, 0.f);
        unsigned long long st = seed * 0x9E3779B97F4A7C15ull + 12345ull;
        auto nrm = [&]() {
            auto nx = [&]() {
                st = st * 6364136223846793005ull + 1442695040888963407ull;
                return ((double)(st >> 11) + 0.5) / 9007199254740992.0;
            };
            const double u1 = nx(), u2 = nx();
            return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        };
        for (int t = 0; t < MLP_H * MLP_IN; t++) p[OW1 + t] = (float)(nrm() * std::sqrt(2.0 / MLP_IN));
        for (int t = 0; t < MLP_H * MLP_H; t++) p[OW2 + t] = (float)(nrm() * std::sqrt(2.0 / MLP_H));
        for (int t = 0; t < MLP_H; t++) p[OW3 + t] = (float)(nrm() * std::sqrt(1.0 / MLP_H));
        PGB_CUDA(cudaMalloc(&M->p, sizeof(float) * MLP_NP));
        PGB_CUDA(cudaMalloc(&M->g, sizeof(float) * MLP_NP));
        PGB_CUDA(cudaMalloc(&M->m1, sizeof(float) * MLP_NP));
        PGB_CUDA(cudaMalloc(&M->m2, sizeof(float) * MLP_NP));
        PGB_CUDA(cudaMemcpy(M->p, p.data(), sizeof(float) * MLP_NP, cudaMemcpyHostToDevice));
        PGB_CUDA(cudaMemset(M->g, 0, sizeof(float) * MLP_NP));
        PGB_CUDA(cudaMemset(M->m1, 0, sizeof(float) * MLP_NP));
        PGB_CUDA(cudaMemset(M->m2, 0, sizeof(float) * MLP_NP));
        PGB_CUDA(cudaMalloc(&M->W1b, sizeof(bf16) * MLP_H * MLP_IN));
        PGB_CUDA(cudaMalloc(&M->W2b, sizeof(bf16) * MLP_H * MLP_H));
        PGB_CUDA(cudaMalloc(&M->W2Tb, sizeof(bf16) * MLP_H * MLP_H));
        PGB_CUDA(cudaMalloc(&M->w3b, sizeof(bf16) * MLP_H));
        const size_t red = std::max<size_t>((size_t)MLP_GRID * (MLP_H * (MLP_IN + 1)) * sizeof(float),
                                            (size_t)MLP_GRID * 4096 * sizeof(double));
        PGB_CUDA(cudaMalloc(&M->red, red));
        PGB_CUDA(cudaMalloc(&M->coef, sizeof(double) * 4096));
        PGB_CUDA(cudaMalloc(&M->part, sizeof(float) * (size_t)MLP_DW2_CHUNKS * (MLP_H * MLP_H + MLP_H)));
        PGB_CUDA(cudaFuncSetAttribute(k_mlp_mm<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mm_smem()));
        PGB_CUDA(cudaFuncSetAttribute(k_mlp_mm<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mm_smem()));
        PGB_CUDA(cudaFuncSetAttribute(k_mlp_mm_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, TM_SMEM));
        PGB_CUDA(cudaFuncSetAttribute(k_mlp_mm_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TM_SMEM));
        PGB_CUDA(cudaMalloc(&M->err, sizeof(int)));
        PGB_CUDA(cudaMemset(M->err, 0, sizeof(int)));
        mlp_cast(*M);
        PGB_CUDA(cudaStreamSynchronize(M->s));
        std::lock_guard<std::mutex> lk(g_mlp_mu);
        *handle = g_mlp_next++;
        g_mlps[*handle] = M;
    })
}

extern "C" int propack_mlp_destroy(int64_t handle)
{
    Mlp *M = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mlp_mu);
        auto it = g_mlps.find(handle);
        if (it == g_mlps.end()) return PROPACK_ERR_HANDLE;
        M = it->second;
        g_mlps.erase(it);
    }
    cudaStreamSynchronize(M->s);
    for (void *q : {(void *)M->p, (void *)M->g, (void *)M->m1, (void *)M->m2, (void *)M->W1b, (void *)M->W2b,
                    (void *)M->W2Tb, (void *)M->w3b, (void *)M->F, (void *)M->out, (void *)M->gout, (void *)M->D1,
                    (void *)M->H1, (void *)M->H2, (void *)M->D2, (void *)M->Y, (void *)M->om, (void *)M->U,
                    (void *)M->red, (void *)M->coef, (void *)M->part, (void *)M->err})
        if (q) cudaFree(q);
    cudaStreamDestroy(M->s);
    delete M;
    return 0;
}

extern "C" int propack_mlp_params(int64_t handle, float *get, const float *set)
{
    Mlp *M = lookup_mlp(handle);
    if (!M) return PROPACK_ERR_HANDLE;
    MLP_TRY({
        if (set) {
            PGB_CUDA(cudaMemcpyAsync(M->p, set, sizeof(float) * MLP_NP, cudaMemcpyHostToDevice, M->s));
            mlp_cast(*M);
        }
        if (get) PGB_CUDA(cudaMemcpyAsync(get, M->p, sizeof(float) * MLP_NP, cudaMemcpyDeviceToHost, M->s));
        PGB_CUDA(cudaStreamSynchronize(M->s));
    })
}

extern "C" int propack_mlp_nparams(void) { return MLP_NP; }

extern "C" int propack_mlp_set_impl(int impl)
{
    if (impl != 0 && impl != 1) return PROPACK_ERR_ARG;
    g_mlp_impl.store(impl);
    return 0;
}

extern "C" int propack_mlp_features(int64_t handle, int64_t op_handle, uint64_t seed, float *F)
{
    Mlp *M = lookup_mlp(handle);
    if (!M) return PROPACK_ERR_HANDLE;
    MLP_TRY({
        const Operator *op = mlp_operator(op_handle);
        mlp_features(*M, *op, seed);
        if (F) PGB_CUDA(cudaMemcpyAsync(F, M->F, sizeof(float) * (size_t)op->m * MLP_IN, cudaMemcpyDeviceToHost, M->s));
        PGB_CUDA(cudaStreamSynchronize(M->s));
    })
}

extern "C" int propack_mlp_start(int64_t handle, int64_t op_handle, uint64_t seed, double *u0)
{
    Mlp *M = lookup_mlp(handle);
    if (!M) return PROPACK_ERR_HANDLE;
    MLP_TRY({
        if (!u0) { set_error("propack_mlp_start: null output"); throw ArgFailure(); }
        const Operator *op = mlp_operator(op_handle);
        const int m = op->m;
        mlp_features(*M, *op, seed);
        mlp_forward(*M, m);
        std::vector<float> o(m);
        PGB_CUDA(cudaMemcpyAsync(o.data(), M->out, sizeof(float) * m, cudaMemcpyDeviceToHost, M->s));
        PGB_CUDA(cudaStreamSynchronize(M->s));
        mlp_check(*M);
        for (int i = 0; i < m; i++) u0[i] = o[i];
    })
}

// gradient of the loss for (operator, U) without an update; grad: MLP_NP floats
extern "C" int propack_mlp_grad(int64_t handle, int64_t op_handle, uint64_t seed, const double *U, int ldu, int k,
                                float *grad, double *loss)
{
    Mlp *M = lookup_mlp(handle);
    if (!M) return PROPACK_ERR_HANDLE;
    MLP_TRY({
        const Operator *op = mlp_operator(op_handle);
        const int m = op->m;
        if (!U || ldu < m || k < 1 || k > 4000) { set_error("propack_mlp_grad: invalid U"); throw ArgFailure(); }
        mlp_features(*M, *op, seed);
        mlp_reserve(*M, m, k);
        PGB_CUDA(cudaMemcpy2DAsync(M->U, sizeof(double) * m, U, sizeof(double) * ldu, sizeof(double) * m, k,
                                   cudaMemcpyHostToDevice, M->s));
        mlp_forward(*M, m);
        const double L = mlp_backward(*M, m, k);
        if (loss) *loss = L;
        if (grad) PGB_CUDA(cudaMemcpyAsync(grad, M->g, sizeof(float) * MLP_NP, cudaMemcpyDeviceToHost, M->s));
        PGB_CUDA(cudaStreamSynchronize(M->s));
        mlp_check(*M);
    })
}

// one Adam step on (operator, U)
extern "C" int propack_mlp_train_step(int64_t handle, int64_t op_handle, uint64_t seed, const double *U, int ldu,
                                      int k, double lr, double *loss)
{
    Mlp *M = lookup_mlp(handle);
    if (!M) return PROPACK_ERR_HANDLE;
    MLP_TRY({
        const Operator *op = mlp_operator(op_handle);
        const int m = op->m;
        if (!U || ldu < m || k < 1 || k > 4000) { set_error("propack_mlp_train_step: invalid U"); throw ArgFailure(); }
        mlp_features(*M, *op, seed);
        mlp_reserve(*M, m, k);
        PGB_CUDA(cudaMemcpy2DAsync(M->U, sizeof(double) * m, U, sizeof(double) * ldu, sizeof(double) * m, k,
                                   cudaMemcpyHostToDevice, M->s));
        mlp_forward(*M, m);
        const double L = mlp_backward(*M, m, k);
        if (loss) *loss = L;
        M->step++;
        const float c1 = 1.f - std::pow(0.9f, (float)M->step), c2 = 1.f - std::pow(0.999f, (float)M->step);
        k_mlp_adam<<<(MLP_NP + 255) / 256, 256, 0, M->s>>>(M->p, M->g, M->m1, M->m2, (float)lr, c1, c2);
        PGB_LAUNCHED();
        mlp_cast(*M);
        PGB_CUDA(cudaStreamSynchronize(M->s));
        mlp_check(*M);
    })
}
