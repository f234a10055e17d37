// pgb_gemm_tc.cu -- FP64 C = A op(B) on the BF16 tensor cores by an
// error-free split (Ozaki, Ogita, Oishi & Rump 2012, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication"), for the restart and Ritz products of the IRL
// (dlansvd_irl.F:371-398, dritzvec.F:130-198): A is the tall Lanczos basis
// (m x K, K <= OZ_KMAX), B the small FP64 factor.
//
// Every row i of A is written as 2^{E_i} sum_p a_p 2^{-7(p+1)} with OZ_S
// balanced 7-bit integer digits a_p (|a_0| <= 128, |a_p| <= 64), every
// column j of op(B) likewise with exponent F_j; digits are exact in BF16.
// Then
//
//   (A op(B))_ij = 2^{E_i + F_j - 14} sum_g 2^{-7g} T_g,
//   T_g = sum_{p+q=g} sum_l a_p(i,l) b_q(l,j)
//
// and each T_g (g < OZ_S; the dropped levels sit below 2^-56 of the row and
// column scales) is an integer below 2^24 in magnitude, so the FP32
// accumulation of the tensor core is exact.  The levels are combined in
// int64 and the FP64 result is assembled from its bits with integer
// operations (oz_levels), so the FP64 pipe (two lanes per clock per SM)
// does no work per output at all.
//
// The digits of A are produced in registers from the FP64 bits with integer
// operations, straight into mma.sync fragments (m16n8k16, row.col); the
// digits of B come from a small pre-pass and are staged in shared memory.
#include <atomic>
#include <algorithm>

#include "../../include/propack_gb300.h"
#include "pgb.cuh"

namespace pgb {

constexpr int OZ_S = 7;      // digits per operand
constexpr int OZ_KMAX = 256; // keeps every level sum below 2^24
constexpr int OZ_BN = 32;    // columns per CTA (four n8 tiles per warp)
constexpr int OZ_WARPS = 4;  // 16 rows each

// balanced base-128 digits of x relative to 2^E (|x| < 2^E), most
// significant first; integer operations only
__device__ __forceinline__ void oz_digits(double x, int E, int d[OZ_S])
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7ff);
    unsigned long long M = 0;
    if (ex != 0) {
        const unsigned long long m = (bits & ((1ull << 52) - 1)) | (1ull << 52);
        const int sh = (ex - 1075) + 7 * OZ_S - E;  // M = m 2^sh < 2^{7 OZ_S}
        if (sh >= 0) M = m << sh;
        else if (sh > -64) M = m >> (-sh);
    }
#pragma unroll
    for (int p = OZ_S - 1; p >= 1; p--) {
        int dd = (int)(M & 127ull);
        M >>= 7;
        if (dd >= 64) { dd -= 128; M += 1; }
        d[p] = dd;
    }
    d[0] = (int)M;
    if (bits >> 63)
#pragma unroll
        for (int p = 0; p < OZ_S; p++) d[p] = -d[p];
}

// small integer (|v| <= 256) -> BF16 bits, exactly, on the FP32 pipe
__device__ __forceinline__ unsigned oz_bf16(int v)
{
    const float f = __int_as_float(0x4B000000 + v + 512) - 8389120.0f;  // 2^23 + 512
    return __float_as_uint(f) >> 16;
}

// max binary exponent E with |x| < 2^E over values (integer compare of the
// exponent fields); -2000 when all are zero
__device__ __forceinline__ int oz_exp_of(double x)
{
    const int ex = (int)(((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff);
    return ex == 0 ? -2000 : ex - 1022;
}

// digits of op(B): Bd[(q * ncp + j) * Kp + l] (BF16 bits), Fe[j]
__global__ void k_oz_bdigits(int kk, int nc, const double *B, int ldb, int tb, int Kp, int ncp,
                             unsigned short *Bd, int *Fe)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncp) return;
    auto bval = [&](int l) -> double { return tb ? B[(size_t)l * ldb + j] : B[(size_t)j * ldb + l]; };
    int E = -2000;
    if (j < nc)
        for (int l = 0; l < kk; l++) E = max(E, oz_exp_of(bval(l)));
    if (E == -2000) E = 0;
    Fe[j] = E;
    for (int l = 0; l < Kp; l++) {
        int d[OZ_S];
        if (j < nc && l < kk) oz_digits(bval(l), E, d);
        else
#pragma unroll
            for (int p = 0; p < OZ_S; p++) d[p] = 0;
#pragma unroll
        for (int q = 0; q < OZ_S; q++) Bd[((size_t)q * ncp + j) * Kp + l] = (unsigned short)oz_bf16(d[q]);
    }
}

__device__ __forceinline__ void mma_bf16(float c[4], const unsigned a[4], unsigned b0, unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// |x| 2^{7 OZ_S - E} as an integer plus OZ_BIAS (64 in every digit below the
// top one), and the sign: balanced digit p is then ((M >> 7 (OZ_S-1-p)) & 127)
// - 64 for p >= 1 and M >> 7 (OZ_S-1) for p = 0
constexpr unsigned long long oz_bias()
{
    unsigned long long b = 0;
    for (int p = 1; p < OZ_S; p++) b = (b << 7) | 64ull;
    return b;
}
constexpr unsigned long long OZ_BIAS = oz_bias();
__device__ __forceinline__ unsigned long long oz_fixed(double x, int E, unsigned &neg)
{
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7ff);
    unsigned long long M = 0;
    if (ex != 0) {
        const unsigned long long m = (bits & ((1ull << 52) - 1)) | (1ull << 52);
        const int sh = (ex - 1075) + 7 * OZ_S - E;
        if (sh >= 0) M = m << sh;
        else if (sh > -64) M = m >> (-sh);
    }
    neg = (unsigned)(bits >> 63);
    return M + OZ_BIAS;
}
template <int P>
__device__ __forceinline__ unsigned oz_digit_bf16(unsigned long long Mb, unsigned neg)
{
    int d = (P == 0) ? (int)(Mb >> (7 * (OZ_S - 1))) : (int)((Mb >> (7 * (OZ_S - 1 - P))) & 127ull) - 64;
    return oz_bf16(neg ? -d : d);
}

// BF16 fragment of A digit P (see k_oz_gemm for the element order)
template <int P>
__device__ __forceinline__ void oz_frag(unsigned (&af)[OZ_S][4], const unsigned long long (&Mb)[8],
                                        const unsigned (&ng)[8])
{
    af[P][0] = oz_digit_bf16<P>(Mb[0], ng[0]) | (oz_digit_bf16<P>(Mb[1], ng[1]) << 16);
    af[P][1] = oz_digit_bf16<P>(Mb[2], ng[2]) | (oz_digit_bf16<P>(Mb[3], ng[3]) << 16);
    af[P][2] = oz_digit_bf16<P>(Mb[4], ng[4]) | (oz_digit_bf16<P>(Mb[5], ng[5]) << 16);
    af[P][3] = oz_digit_bf16<P>(Mb[6], ng[6]) | (oz_digit_bf16<P>(Mb[7], ng[7]) << 16);
}

// V 2^sc as an FP64 value, rounded to nearest even: the bits are assembled
// with integer operations (the same value as ldexp((double)V, sc) whenever
// the result is a normal number; otherwise that general path runs).  This
// keeps the epilogue off the FP64 pipe, which retires two lanes per clock.
__device__ __forceinline__ double oz_compose(long long V, int sc)
{
    if (V == 0) return 0.0;
    const unsigned long long sgn = V < 0 ? (1ull << 63) : 0ull;
    const unsigned long long a = V < 0 ? 0ull - (unsigned long long)V : (unsigned long long)V;
    const int nb = 64 - __clzll((long long)a);  // significant bits of |V|
    int ex = nb - 1 + sc;                       // unbiased exponent of the result
    unsigned long long m;                       // significand with its leading bit
    if (nb <= 53) {
        m = a << (53 - nb);
    } else {
        const int sh = nb - 53;
        m = a >> sh;
        const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (m & 1ull))) m++;
        if (m >> 53) {
            m >>= 1;
            ex++;
        }
    }
    if (ex < -1022 || ex > 1023) return ldexp((double)V, sc);
    return __longlong_as_double((long long)(sgn | ((unsigned long long)(ex + 1023) << 52) | (m & ((1ull << 52) - 1))));
}

// The levels T_0 .. T_6 (exact integers) of one output, scaled by 2^sc:
// sum_g T_g 128^(6-g) 2^sc.  The low levels fit an int64 (|lo| < 2^59); the
// whole sum does while |T_0| < 2^19, which holds unless nearly every
// product of a row and a column has the same sign and the largest size --
// there the two parts are rounded separately.
__device__ __forceinline__ double oz_levels(const int (&T)[OZ_S], int sc)
{
    long long lo = 0;
#pragma unroll
    for (int g = 1; g < OZ_S; g++) lo = lo * 128 + T[g];
    const long long hi = T[0];
    if (hi > -(1ll << 19) && hi < (1ll << 19)) return oz_compose(hi * (1ll << (7 * (OZ_S - 1))) + lo, sc);
    return ldexp((double)hi, sc + 7 * (OZ_S - 1)) + ldexp((double)lo, sc);
}

// C(mr x nc) = A(mr x kk, column-major lda) op(B); one warp per 16 rows and
// OZ_BN columns.  Row fragment positions (m16n8k16): rows gid, gid+8; K
// columns 2 tig + {0, 1, 8, 9}; C columns 2 tig + {0, 1} of each n8 tile.
// Dynamic shared memory: the digits of the CTA's OZ_BN columns of op(B),
// [q][column][Kp].
__global__ void __launch_bounds__(OZ_WARPS * 32) k_oz_gemm(int mr, int nc, int kk, const double *__restrict__ A,
                                                          int lda, const unsigned short *__restrict__ Bd,
                                                          const int *__restrict__ Fe, int Kp, int ncp,
                                                          double *__restrict__ C, int ldc)
{
    extern __shared__ unsigned short Bs[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gid = lane >> 2, tig = lane & 3;
    // the column tiles of one row block are neighbours in the launch order,
    // so the second one finds the A rows in L2
    const int ntc = ncp / OZ_BN;
    const int row0 = ((blockIdx.x / ntc) * OZ_WARPS + w) * 16;
    const int col0 = (blockIdx.x % ntc) * OZ_BN;
    // stage the digits of columns col0 .. col0+OZ_BN-1; rows of KS = Kp + 8
    // elements keep the eight fragment columns of a load on distinct banks
    const int KS = Kp + 8;
    {
        const int wpr = Kp / 2;  // 32-bit words per (digit, column)
        unsigned *dst = reinterpret_cast<unsigned *>(Bs);
        for (int i = threadIdx.x; i < OZ_S * OZ_BN * wpr; i += blockDim.x) {
            const int qj = i / wpr, o = i % wpr;
            const int q = qj / OZ_BN, j = qj % OZ_BN;
            dst[qj * (KS / 2) + o] = reinterpret_cast<const unsigned *>(Bd + ((size_t)q * ncp + col0 + j) * Kp)[o];
        }
    }
    __syncthreads();
    if (row0 >= mr) return;
    // row exponents of rows row0 + gid and row0 + gid + 8 (the lanes of a
    // quad share them): each lane scans every fourth K column
    const int ra = row0 + gid, rb = ra + 8;
    int Ea = -2000, Eb = -2000;
    for (int l = tig; l < kk; l += 4) {
        if (ra < mr) Ea = max(Ea, oz_exp_of(A[(size_t)l * lda + ra]));
        if (rb < mr) Eb = max(Eb, oz_exp_of(A[(size_t)l * lda + rb]));
    }
    Ea = max(Ea, __shfl_xor_sync(0xffffffffu, Ea, 1));
    Ea = max(Ea, __shfl_xor_sync(0xffffffffu, Ea, 2));
    Eb = max(Eb, __shfl_xor_sync(0xffffffffu, Eb, 1));
    Eb = max(Eb, __shfl_xor_sync(0xffffffffu, Eb, 2));
    if (Ea == -2000) Ea = 0;
    if (Eb == -2000) Eb = 0;

    float acc[OZ_S][4][4];
#pragma unroll
    for (int g = 0; g < OZ_S; g++)
#pragma unroll
        for (int t = 0; t < 4; t++)
#pragma unroll
            for (int r = 0; r < 4; r++) acc[g][t][r] = 0.f;

    // fragment elements e: {ra,k}{ra,k+1} {rb,k}{rb,k+1} {ra,k+8}{ra,k+9} {rb,k+8}{rb,k+9};
    // the values of the next K step are loaded while this one computes
    double xv[8];
    auto load_step = [&](int k0) {
#pragma unroll
        for (int h = 0; h < 2; h++)
#pragma unroll
            for (int c = 0; c < 2; c++) {
                const int kc = k0 + 2 * tig + c + 8 * h;
                xv[h * 4 + c] = (kc < kk && ra < mr) ? A[(size_t)kc * lda + ra] : 0.0;
                xv[h * 4 + 2 + c] = (kc < kk && rb < mr) ? A[(size_t)kc * lda + rb] : 0.0;
            }
    };
    load_step(0);
    for (int k0 = 0; k0 < Kp; k0 += 16) {
        unsigned long long Mb[8];
        unsigned ng[8];
#pragma unroll
        for (int e = 0; e < 8; e++) Mb[e] = oz_fixed(xv[e], (e & 2) ? Eb : Ea, ng[e]);
        if (k0 + 16 < Kp) load_step(k0 + 16);
        unsigned af[OZ_S][4];
        oz_frag<0>(af, Mb, ng);
        oz_frag<1>(af, Mb, ng);
        oz_frag<2>(af, Mb, ng);
        oz_frag<3>(af, Mb, ng);
        oz_frag<4>(af, Mb, ng);
        oz_frag<5>(af, Mb, ng);
        oz_frag<6>(af, Mb, ng);
        // each B fragment (tile t, digit q) is loaded once and serves every
        // A digit p with p + q < OZ_S
#pragma unroll
        for (int t = 0; t < 4; t++)
#pragma unroll
            for (int q = 0; q < OZ_S; q++) {
                const unsigned short *bp = Bs + ((size_t)q * OZ_BN + 8 * t + gid) * KS + k0 + 2 * tig;
                const unsigned b0 = *reinterpret_cast<const unsigned *>(bp);
                const unsigned b1 = *reinterpret_cast<const unsigned *>(bp + 8);
#pragma unroll
                for (int p = 0; p + q < OZ_S; p++) mma_bf16(acc[p + q][t], af[p], b0, b1);
            }
    }
    // V = sum_g T_g 2^{7 (OZ_S - 1 - g)};  C = V 2^{E + F - 14 - 7 (OZ_S - 1)}
#pragma unroll
    for (int t = 0; t < 4; t++)
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int row = (r < 2) ? ra : rb;
            const int col = col0 + 8 * t + 2 * tig + (r & 1);
            int T[OZ_S];
#pragma unroll
            for (int g = 0; g < OZ_S; g++) T[g] = __float2int_rn(acc[g][t][r]);
            if (row < mr && col < nc) {
                const int sc = ((r < 2) ? Ea : Eb) + Fe[col] - 14 - 7 * (OZ_S - 1);
                C[(size_t)col * ldc + row] = oz_levels(T, sc);
            }
        }
}

// ===========================================================================
// The same product on the 5th-generation tensor cores: tcgen05.mma with the
// seven level sums T_g accumulated in tensor memory.
//
// One CTA (512 threads, one per SM: its shared memory and 512 TMEM columns
// admit no second) owns 128 rows x UM_BN columns.  K runs in stages of
// UM_KC = 32 (two K = 16 MMA steps), double-buffered: while the tensor core
// works on stage c, the threads load the FP64 values of stage c + 1, split
// them into digits and write the digit planes of A into the other buffer;
// the digit planes of B for the stage arrive by one bulk copy (cp.async.bulk
// into shared memory, completion on an mbarrier).  Per stage, thread 0
// issues 2 x 28 MMAs (M = 128, N = UM_BN, K = 16, BF16 x BF16 -> FP32): the
// digit pair (p, q) of K step s accumulates into the TMEM columns of level
// p + q.  tcgen05.commit arrives on the stage's mbarrier when those MMAs are
// done, which frees the stage's buffers.  After the last stage every warp
// reads its 32 TMEM lanes (rows) with tcgen05.ld and combines the levels
// in int64 as above.
//
// Operand layout in shared memory (no swizzle, K-major): a (digit, K step)
// tile of R rows x 16 K is R/8 x 2 core matrices of 8 rows x 16 bytes; row
// group g, K half h sits at g * 256 + h * 128 bytes (descriptor leading
// byte offset 128 = next core matrix along K, stride byte offset 256 = next
// 8-row group).  Every wait is bounded; a wait that runs out sets *err and
// the CTA skips the rest of its work.
constexpr int UM_BM = 128;
constexpr int UM_BN = 64;
constexpr int UM_KC = 32;
constexpr int UM_THREADS = 512;  // four threads per row: 8 K values of a stage each
constexpr int UM_ATILE = UM_BM * 16 * 2;        // 4096 bytes
constexpr int UM_BTILE = UM_BN * 16 * 2;        // 2048 bytes
constexpr int UM_ASTAGE = OZ_S * 2 * UM_ATILE;  // 57344 bytes
constexpr int UM_BSTAGE = OZ_S * 2 * UM_BTILE;  // 28672 bytes
constexpr int UM_SMEM = 2 * (UM_ASTAGE + UM_BSTAGE) + 4096;
constexpr unsigned UM_TMEM_COLS = 512;          // OZ_S * UM_BN = 448 FP32 columns, rounded up to a power of two
// instruction descriptor (kind::f16): FP32 accumulator, BF16 A and B, both
// K-major, N / 8, M / 16
constexpr uint32_t UM_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(UM_BN >> 3) << 17) |
                              ((uint32_t)(UM_BM >> 4) << 24);
constexpr long UM_WAIT_LIMIT = 1L << 22;
static_assert(OZ_S * UM_BN <= (int)UM_TMEM_COLS, "levels must fit in TMEM");
static_assert(UM_SMEM <= 227 * 1024, "shared memory");

__device__ __forceinline__ uint32_t um_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared memory matrix descriptor: start address, LBO 128 B, SBO 256 B,
// the fixed 0b001 at bits 46-48, no swizzle
__device__ __forceinline__ uint64_t um_desc(uint32_t saddr)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
           (1ull << 46);
}
__device__ __forceinline__ void um_bar_init(uint32_t bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool um_bar_try(uint32_t bar, unsigned parity)
{
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool um_bar_wait(uint32_t bar, unsigned parity)
{
    for (long it = 0; it < UM_WAIT_LIMIT; it++)
        if (um_bar_try(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void um_st16(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}
__device__ __forceinline__ void um_mma(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t acc)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
        "l"(ad), "l"(bd), "r"(UM_IDESC), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void um_ld8(uint32_t taddr, uint32_t (&v)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
                 : "r"(taddr)
                 : "memory");
}

// digit P of a value in the biased fixed-point form of oz_fixed, as FP32
// bits (exact: |digit| <= 128): the 7-bit field OR'd into the mantissa of
// 2^23, then one FMA removes 2^23 (and the bias 64 below the top digit)
// and applies the sign sg = +-1
template <int P>
__device__ __forceinline__ uint32_t um_digit(unsigned long long Mb, float sg)
{
    const unsigned field = P == 0 ? (unsigned)(Mb >> (7 * (OZ_S - 1)))
                                  : ((unsigned)(Mb >> (7 * (OZ_S - 1 - P))) & 127u);
    const float off = P == 0 ? -8388608.0f : -8388672.0f;
    return __float_as_uint(fmaf(sg, __uint_as_float(field | 0x4B000000u), sg * off));
}

// the eight digits P of this thread's K values -> one 16-byte core-matrix row
template <int P>
__device__ __forceinline__ void um_plane(uint32_t arow, const unsigned long long (&Mb)[8], const float (&sg)[8])
{
    uint32_t w[4];
#pragma unroll
    for (int j = 0; j < 4; j++)
        w[j] = __byte_perm(um_digit<P>(Mb[2 * j], sg[2 * j]), um_digit<P>(Mb[2 * j + 1], sg[2 * j + 1]), 0x7632);
    um_st16(arow + P * 2 * UM_ATILE, w[0], w[1], w[2], w[3]);
}

// digit planes of op(B) in the shared-memory image of every (column tile,
// stage): [tile][stage][q][K step][UM_BTILE], and the column exponents
__global__ void k_oz_bimg(int kk, int nc, const double *B, int ldb, int tb, int ntc, int nstage,
                          unsigned short *img, int *Fe)
{
    const int jg = blockIdx.x * blockDim.x + threadIdx.x;
    if (jg >= ntc * UM_BN) return;
    auto bval = [&](int l) -> double { return tb ? B[(size_t)l * ldb + jg] : B[(size_t)jg * ldb + l]; };
    int E = -2000;
    if (jg < nc)
        for (int l = 0; l < kk; l++) E = max(E, oz_exp_of(bval(l)));
    if (E == -2000) E = 0;
    Fe[jg] = E;
    const int ct = jg / UM_BN, j = jg % UM_BN;
    for (int l = 0; l < nstage * UM_KC; l++) {
        int d[OZ_S];
        if (jg < nc && l < kk) oz_digits(bval(l), E, d);
        else
#pragma unroll
            for (int p = 0; p < OZ_S; p++) d[p] = 0;
        const int c = l / UM_KC, st = (l % UM_KC) / 16, k = l % 16;
        const size_t base = ((size_t)ct * nstage + c) * UM_BSTAGE + (size_t)((j >> 3) * 256 + (k >> 3) * 128 +
                                                                             (j & 7) * 16 + (k & 7) * 2);
#pragma unroll
        for (int q = 0; q < OZ_S; q++) img[(base + (size_t)(q * 2 + st) * UM_BTILE) / 2] = (unsigned short)oz_bf16(d[q]);
    }
}

// Persistent: CTA b takes the tiles b, b + grid, ... (tile = row block x
// column tile, column tiles fastest).  While a tile's stages run, every
// thread also loads sixteen values of its row of the CTA's next tile per
// stage and keeps their largest exponent, so the next tile's row scales
// are ready when it starts (and its values sit in L2).
__global__ void __launch_bounds__(UM_THREADS, 1) k_oz_umma(int mr, int nc, int kk, const double *__restrict__ A, int lda,
                                                          const unsigned short *__restrict__ Bimg,
                                                          const int *__restrict__ Fe, int nstage,
                                                          double *__restrict__ C, int ldc, int *err)
{
    extern __shared__ __align__(1024) unsigned char um_sm[];
    unsigned char *As = um_sm;
    unsigned char *Bs = um_sm + 2 * UM_ASTAGE;
    uint64_t *bar = reinterpret_cast<uint64_t *>(Bs + 2 * UM_BSTAGE);  // [0..1] B copies, [2..3] MMAs
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 4);
    int *sbad = reinterpret_cast<int *>(tslot + 1);
    int *Ep = reinterpret_cast<int *>(tslot + 4);  // [4][UM_BM]
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int ntc = (nc + UM_BN - 1) / UM_BN;
    const int ntiles = (mr + UM_BM - 1) / UM_BM * ntc;
    const uint32_t a_s = um_smem(As), b_s = um_smem(Bs), bar_s = um_smem(bar);
    if (tid == 0) {
        for (int i = 0; i < 4; i++) um_bar_init(bar_s + 8 * i, 1);
        *sbad = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(um_smem(tslot)),
                     "r"(UM_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // thread (r, h): row r of the tile; K values 8 h .. 8 h + 7 of every
    // stage (K step h / 2, its half h % 2); K columns h, h + 4, ... of the
    // exponent scans
    const int r = tid & (UM_BM - 1), h = tid >> 7;
    auto tile_row = [&](int t) { return (t / ntc) * UM_BM + r; };
    // the eight scan values of stage c of tile t (columns h + 4 (8 c + u))
    auto scan_load = [&](int t, int c, double (&sv)[8]) {
        const int row = tile_row(t);
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int l = h + 4 * (8 * c + u);
            sv[u] = (t < ntiles && row < mr && l < kk) ? A[(size_t)l * lda + row] : 0.0;
        }
    };
    auto scan_fold = [&](int &Eacc, const double (&sv)[8]) {
#pragma unroll
        for (int u = 0; u < 8; u++) Eacc = max(Eacc, oz_exp_of(sv[u]));
    };
    // the eight stage values of stage c of tile t
    double xv[8];
    auto load_stage = [&](int t, int c) {
        const int row = tile_row(t), k0 = c * UM_KC + h * 8;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int l = k0 + i;
            xv[i] = (t < ntiles && row < mr && l < kk) ? A[(size_t)l * lda + row] : 0.0;
        }
    };
    // row scales of the CTA's first tile: a plain scan
    int t = blockIdx.x;
    int E = -2000;
    for (int c = 0; c < nstage; c++) {
        double sv[8];
        scan_load(t, c, sv);
        scan_fold(E, sv);
    }
    Ep[h * UM_BM + r] = E;
    load_stage(t, 0);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    E = max(max(Ep[r], Ep[UM_BM + r]), max(Ep[2 * UM_BM + r], Ep[3 * UM_BM + r]));
    if (E == -2000) E = 0;
    __syncthreads();  // Ep is written again at the end of the first tile

    const uint32_t arow_off = (uint32_t)((h >> 1) * UM_ATILE + (r >> 3) * 256 + (h & 1) * 128 + (r & 7) * 16);
    int g = 0;  // stages issued so far by this CTA (mbarrier phases)
    bool bad = false;
    for (; t < ntiles && !bad; t += gridDim.x) {
        const int tn = t + gridDim.x;
        const int ct = t % ntc, col0 = ct * UM_BN, row0 = (t / ntc) * UM_BM;
        int En = -2000;
        double sv[8];
        for (int c = 0; c < nstage; c++, g++) {
            const int b = g & 1;
            bool ok = true;
            if (g >= 2) ok = um_bar_wait(bar_s + 8 * (2 + b), ((g - 2) >> 1) & 1);  // MMAs of stage g - 2 done
            if (__syncthreads_or(!ok || *sbad)) {
                bad = true;
                break;
            }
            if (c > 0) scan_fold(En, sv);
            if (tid == 0) {
                const uint32_t tb_ = bar_s + 8 * b;
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tb_), "r"(UM_BSTAGE)
                             : "memory");
                const unsigned short *src = Bimg + ((size_t)ct * nstage + c) * (UM_BSTAGE / 2);
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        b_s + b * UM_BSTAGE),
                    "l"(src), "r"(UM_BSTAGE), "r"(tb_)
                    : "memory");
            }
            unsigned long long Mb[8];
            float sg[8];
#pragma unroll
            for (int i = 0; i < 8; i++) {
                unsigned ng;
                Mb[i] = oz_fixed(xv[i], E, ng);
                sg[i] = ng ? -1.0f : 1.0f;
            }
            // the next stage's values (this tile's, or the next tile's first)
            if (c + 1 < nstage) load_stage(t, c + 1);
            else load_stage(tn, 0);
            scan_load(tn, c, sv);
            const uint32_t arow = a_s + b * UM_ASTAGE + arow_off;
            um_plane<0>(arow, Mb, sg);
            um_plane<1>(arow, Mb, sg);
            um_plane<2>(arow, Mb, sg);
            um_plane<3>(arow, Mb, sg);
            um_plane<4>(arow, Mb, sg);
            um_plane<5>(arow, Mb, sg);
            um_plane<6>(arow, Mb, sg);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (tid == 0) {
                if (!um_bar_wait(bar_s + 8 * b, (g >> 1) & 1)) {
                    *sbad = 1;
                } else {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    // descriptors differ only in the start address field (the
                    // low 14 bits, which no tile offset here carries out of)
                    const uint64_t ad0 = um_desc(a_s + b * UM_ASTAGE), bd0 = um_desc(b_s + b * UM_BSTAGE);
#pragma unroll
                    for (int st = 0; st < 2; st++)
#pragma unroll
                        for (int p = 0; p < OZ_S; p++)
#pragma unroll
                            for (int q = 0; p + q < OZ_S; q++)
                                um_mma(tmem + (uint32_t)((p + q) * UM_BN), ad0 + (uint64_t)(((p * 2 + st) * UM_ATILE) >> 4),
                                       bd0 + (uint64_t)(((q * 2 + st) * UM_BTILE) >> 4),
                                       (c == 0 && st == 0 && p == 0) ? 0u : 1u);
                    asm volatile(
                        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                            bar_s + 8 * (2 + b))
                        : "memory");
                }
            }
        }
        if (bad) break;
        // every MMA of the tile is covered by its last stage's commit
        const int gl = g - 1;
        const bool ok = !*sbad && um_bar_wait(bar_s + 8 * (2 + (gl & 1)), (gl >> 1) & 1);
        if (__syncthreads_or(!ok)) {
            bad = true;
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        scan_fold(En, sv);
        Ep[h * UM_BM + r] = En;
        {
            // warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows), columns
            // 16 (w / 4) .. + 15 in two halves of 8
            const int L = 32 * (w & 3), hc = w >> 2;
            const int orow = row0 + L + lane;  // this thread's row r
#pragma unroll
            for (int ph = 0; ph < 2; ph++) {
                const int cb = hc * 16 + ph * 8;
                uint32_t v[OZ_S][8];
#pragma unroll
                for (int gg = 0; gg < OZ_S; gg++)
                    um_ld8(tmem + ((uint32_t)L << 16) + (uint32_t)(gg * UM_BN + cb), v[gg]);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int jj = 0; jj < 8; jj++) {
                    const int col = col0 + cb + jj;
                    int T[OZ_S];
#pragma unroll
                    for (int gg = 0; gg < OZ_S; gg++) T[gg] = __float2int_rn(__uint_as_float(v[gg][jj]));
                    if (orow < mr && col < nc)
                        C[(size_t)col * ldc + orow] = oz_levels(T, E + Fe[col] - 14 - 7 * (OZ_S - 1));
                }
            }
        }
        // the TMEM reads and the exponent halves are done before the next
        // tile's first MMAs overwrite the levels
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        E = max(max(Ep[r], Ep[UM_BM + r]), max(Ep[2 * UM_BM + r], Ep[3 * UM_BM + r]));
        if (E == -2000) E = 0;
        __syncthreads();
    }
    if (bad && tid == 0) atomicExch(err, 1);
    if (bad && g > 0) {
        // let the MMAs in flight finish (bounded) before the columns are freed
        const int gl = g - 1;
        um_bar_wait(bar_s + 8 * (2 + (gl & 1)), (gl >> 1) & 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (w == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(UM_TMEM_COLS) : "memory");
}

// ===========================================================================
// The same product, warp-specialised.  Sixteen producer warps (four threads
// per row, as above) split A into digit planes; one more warp, the MMA warp,
// copies B's digit planes in (cp.async.bulk) and issues the MMAs.  The two
// roles meet only on mbarriers, so no CTA-wide barrier sits between a
// stage's digits and its MMAs:
//
//   full[b]   the producers' 512 arrivals: stage buffer b holds its A digits
//             (each thread fences its shared-memory writes into the async
//             proxy first)
//   bfull[b]  the bulk copy of B's digits for the stage in buffer b landed
//   empty[b]  tcgen05.commit of the stage's MMAs: buffer b may be rewritten
//   tfull     tcgen05.commit after a tile's last stage: TMEM holds its levels
//   tempty    the producers' 512 arrivals after reading TMEM: the next
//             tile's first MMAs may overwrite the levels
//
// Stage g uses buffer g % 2, phase (g / 2) % 2 of full/bfull/empty; tile tt
// (of this CTA) phase tt % 2 of tfull/tempty.  No barrier can run two phases
// ahead of its waiter: refilling a buffer waits for the MMAs that read it,
// which wait for the fill before.  Every wait is bounded; a wait that runs
// out sets the CTA's flag, which every loop checks, and the kernel reports
// it through *err after the MMAs in flight have finished (bounded) and the
// tensor memory is freed.  The row exponents of the next tile are folded
// into the current tile's stages as above and exchanged among the producers
// only (named barrier 1).  Results are bit-identical to k_oz_umma.
constexpr int WS_PROD = 512;              // producer threads
constexpr int WS_THREADS = WS_PROD + 32;  // + the MMA warp
__device__ __forceinline__ void ws_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void ws_prod_sync() { asm volatile("bar.sync 1, %0;" ::"n"(WS_PROD) : "memory"); }
// a barrier of the producers only that also ORs a flag over them
__device__ __forceinline__ bool ws_prod_or(bool v)
{
    uint32_t r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 p, %1, 0;\nbar.red.or.pred q, 1, %2, p;\nselp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(WS_PROD)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ bool ws_bad(const int *sbad) { return *(volatile const int *)sbad != 0; }
// bounded wait that gives up early once the CTA's flag is set
__device__ __forceinline__ bool ws_wait(uint32_t bar, unsigned parity, int *sbad)
{
    for (long it = 0; it < UM_WAIT_LIMIT; it++) {
        if (um_bar_try(bar, parity)) return true;
        if ((it & 255) == 255 && ws_bad(sbad)) return false;
    }
    *(volatile int *)sbad = 1;
    return false;
}

__global__ void __launch_bounds__(WS_THREADS, 1) k_oz_umma_ws(int mr, int nc, int kk, const double *__restrict__ A,
                                                             int lda, const unsigned short *__restrict__ Bimg,
                                                             const int *__restrict__ Fe, int nstage,
                                                             double *__restrict__ C, int ldc, int *err)
{
    extern __shared__ __align__(1024) unsigned char um_sm[];
    unsigned char *As = um_sm;
    unsigned char *Bs = um_sm + 2 * UM_ASTAGE;
    uint64_t *bar = reinterpret_cast<uint64_t *>(Bs + 2 * UM_BSTAGE);
    // [0..1] full, [2..3] bfull, [4..5] empty, [6] tfull, [7] tempty
    uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 8);
    int *sbad = reinterpret_cast<int *>(tslot + 1);
    int *Ep = reinterpret_cast<int *>(tslot + 4);  // [4][UM_BM]
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int ntc = (nc + UM_BN - 1) / UM_BN;
    const int ntiles = (mr + UM_BM - 1) / UM_BM * ntc;
    const uint32_t a_s = um_smem(As), b_s = um_smem(Bs), bar_s = um_smem(bar);
    const uint32_t FULL = bar_s, BFULL = bar_s + 16, EMPTY = bar_s + 32, TFULL = bar_s + 48, TEMPTY = bar_s + 56;
    if (tid == 0) {
        um_bar_init(FULL, WS_PROD);
        um_bar_init(FULL + 8, WS_PROD);
        um_bar_init(BFULL, 1);
        um_bar_init(BFULL + 8, 1);
        um_bar_init(EMPTY, 1);
        um_bar_init(EMPTY + 8, 1);
        um_bar_init(TFULL, 1);
        um_bar_init(TEMPTY, WS_PROD);
        *sbad = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (w == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(um_smem(tslot)),
                     "r"(UM_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;

    if (tid >= WS_PROD) {
        // ------------------------------------------------------ MMA warp
        if (lane == 0) {
            int g = 0, tt = 0;
            // the bulk copy of B's digits for stage g (tile t, stage c) into buffer g % 2
            auto copy_b = [&](int t, int c, int gg) {
                const uint32_t bb = BFULL + 8 * (gg & 1);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bb), "r"(UM_BSTAGE)
                             : "memory");
                const unsigned short *src = Bimg + ((size_t)(t % ntc) * nstage + c) * (UM_BSTAGE / 2);
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        b_s + (gg & 1) * UM_BSTAGE),
                    "l"(src), "r"(UM_BSTAGE), "r"(bb)
                    : "memory");
            };
            // stage after (t, c): (t, c + 1) or (t + grid, 0)
            auto next_stage = [&](int &t, int &c) {
                if (++c == nstage) {
                    c = 0;
                    t += gridDim.x;
                }
            };
            int tb = blockIdx.x, cb = 0;  // the stage whose B copy goes out next (stage g + 1 in the loop)
            if (tb < ntiles) {
                copy_b(tb, cb, 0);
                next_stage(tb, cb);
            }
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, tt++) {
                if (tt > 0 && !ws_wait(TEMPTY, (tt - 1) & 1, sbad)) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                for (int c = 0; c < nstage; c++, g++) {
                    const int b = g & 1;
                    if (!ws_wait(FULL + 8 * b, (g >> 1) & 1, sbad) || !ws_wait(BFULL + 8 * b, (g >> 1) & 1, sbad)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint64_t ad0 = um_desc(a_s + b * UM_ASTAGE), bd0 = um_desc(b_s + b * UM_BSTAGE);
#pragma unroll
                    for (int st = 0; st < 2; st++)
#pragma unroll
                        for (int p = 0; p < OZ_S; p++)
#pragma unroll
                            for (int q = 0; p + q < OZ_S; q++)
                                um_mma(tmem + (uint32_t)((p + q) * UM_BN),
                                       ad0 + (uint64_t)(((p * 2 + st) * UM_ATILE) >> 4),
                                       bd0 + (uint64_t)(((q * 2 + st) * UM_BTILE) >> 4),
                                       (c == 0 && st == 0 && p == 0) ? 0u : 1u);
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     EMPTY + 8 * b)
                                 : "memory");
                    if (c == nstage - 1)
                        asm volatile(
                            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(TFULL)
                            : "memory");
                    // the other buffer is free once stage g - 1's MMAs are done
                    // (issued before this stage's): the B copy of stage g + 1
                    // goes into it
                    if (tb < ntiles) {
                        if (g >= 1 && !ws_wait(EMPTY + 8 * (b ^ 1), ((g - 1) >> 1) & 1, sbad)) {
                            ok = false;
                            break;
                        }
                        copy_b(tb, cb, g + 1);
                        next_stage(tb, cb);
                    }
                }
            }
            if (!ok) *(volatile int *)sbad = 1;
            // the MMAs issued last are done before the columns are freed
            if (g > 0) um_bar_wait(EMPTY + 8 * ((g - 1) & 1), ((g - 1) >> 1) & 1);
        }
        __syncwarp();
    } else {
        // ------------------------------------------------ producer warps
        const int r = tid & (UM_BM - 1), h = tid >> 7;
        auto tile_row = [&](int t) { return (t / ntc) * UM_BM + r; };
        auto scan_load = [&](int t, int c, double (&sv)[8]) {
            const int row = tile_row(t);
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int l = h + 4 * (8 * c + u);
                sv[u] = (t < ntiles && row < mr && l < kk) ? A[(size_t)l * lda + row] : 0.0;
            }
        };
        auto scan_fold = [&](int &Eacc, const double (&sv)[8]) {
#pragma unroll
            for (int u = 0; u < 8; u++) Eacc = max(Eacc, oz_exp_of(sv[u]));
        };
        double xv[8];
        auto load_stage = [&](int t, int c) {
            const int row = tile_row(t), k0 = c * UM_KC + h * 8;
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int l = k0 + i;
                xv[i] = (t < ntiles && row < mr && l < kk) ? A[(size_t)l * lda + row] : 0.0;
            }
        };
        int t = blockIdx.x;
        int E = -2000;
        for (int c = 0; c < nstage; c++) {
            double sv[8];
            scan_load(t, c, sv);
            scan_fold(E, sv);
        }
        Ep[h * UM_BM + r] = E;
        load_stage(t, 0);
        ws_prod_sync();
        E = max(max(Ep[r], Ep[UM_BM + r]), max(Ep[2 * UM_BM + r], Ep[3 * UM_BM + r]));
        if (E == -2000) E = 0;
        ws_prod_sync();  // Ep is written again at the end of the first tile
        const uint32_t arow_off = (uint32_t)((h >> 1) * UM_ATILE + (r >> 3) * 256 + (h & 1) * 128 + (r & 7) * 16);
        // Control flow is the same in every producer thread (the named
        // barriers need all of them): a wait that fails marks the thread,
        // which then skips its TMEM reads and stores, and the producers stop
        // together at the end of the tile
        int g = 0, tt = 0;
        bool ok = true;
        for (; t < ntiles; t += gridDim.x, tt++) {
            const int tn = t + gridDim.x;
            const int col0 = (t % ntc) * UM_BN, row0 = (t / ntc) * UM_BM;
            int En = -2000;
            double sv[8];
            for (int c = 0; c < nstage; c++, g++) {
                const int b = g & 1;
                if (g >= 2 && ok && !ws_wait(EMPTY + 8 * b, ((g - 2) >> 1) & 1, sbad)) ok = false;
                if (c > 0) scan_fold(En, sv);
                unsigned long long Mb[8];
                float sg[8];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    unsigned ng;
                    Mb[i] = oz_fixed(xv[i], E, ng);
                    sg[i] = ng ? -1.0f : 1.0f;
                }
                if (c + 1 < nstage) load_stage(t, c + 1);
                else load_stage(tn, 0);
                scan_load(tn, c, sv);
                const uint32_t arow = a_s + b * UM_ASTAGE + arow_off;
                um_plane<0>(arow, Mb, sg);
                um_plane<1>(arow, Mb, sg);
                um_plane<2>(arow, Mb, sg);
                um_plane<3>(arow, Mb, sg);
                um_plane<4>(arow, Mb, sg);
                um_plane<5>(arow, Mb, sg);
                um_plane<6>(arow, Mb, sg);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                ws_arrive(FULL + 8 * b);
            }
            if (ok && !ws_wait(TFULL, tt & 1, sbad)) ok = false;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            scan_fold(En, sv);
            Ep[h * UM_BM + r] = En;
            if (ok) {
                const int L = 32 * (w & 3), hc = w >> 2;
                const int orow = row0 + L + lane;
#pragma unroll
                for (int ph = 0; ph < 2; ph++) {
                    const int cb = hc * 16 + ph * 8;
                    uint32_t v[OZ_S][8];
#pragma unroll
                    for (int gg = 0; gg < OZ_S; gg++)
                        um_ld8(tmem + ((uint32_t)L << 16) + (uint32_t)(gg * UM_BN + cb), v[gg]);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                    for (int jj = 0; jj < 8; jj++) {
                        const int col = col0 + cb + jj;
                        int T[OZ_S];
#pragma unroll
                        for (int gg = 0; gg < OZ_S; gg++) T[gg] = __float2int_rn(__uint_as_float(v[gg][jj]));
                        if (orow < mr && col < nc)
                            C[(size_t)col * ldc + orow] = oz_levels(T, E + Fe[col] - 14 - 7 * (OZ_S - 1));
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            ws_arrive(TEMPTY);
            const bool stop = ws_prod_or(!ok || ws_bad(sbad));
            E = max(max(Ep[r], Ep[UM_BM + r]), max(Ep[2 * UM_BM + r], Ep[3 * UM_BM + r]));
            if (E == -2000) E = 0;
            if (stop) break;
        }
        if (!ok) *(volatile int *)sbad = 1;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0 && *sbad) atomicExch(err, 1);
    if (w == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(UM_TMEM_COLS) : "memory");
}

// scratch for the digits of B (grown on demand, per host thread)
struct OzScratch {
    unsigned short *bd = nullptr;
    int *fe = nullptr;
    int *err = nullptr;
    int *herr = nullptr;
    size_t cap = 0, fecap = 0;
    int dev = -1;
    ~OzScratch()
    {
        if (bd) cudaFree(bd);
        if (fe) cudaFree(fe);
        if (err) cudaFree(err);
        if (herr) cudaFreeHost(herr);
    }
};

// need: digit elements of B; nfe: column exponents
static void oz_scratch(OzScratch &sc, size_t need, int nfe)
{
    int dev = 0;
    PGB_CUDA(cudaGetDevice(&dev));
    if (sc.cap < need || sc.fecap < (size_t)nfe || sc.dev != dev) {
        if (sc.bd) {
            PGB_CUDA(cudaDeviceSynchronize());
            cudaFree(sc.bd);
            cudaFree(sc.fe);
            sc.bd = nullptr;
            sc.fe = nullptr;
        }
        sc.cap = std::max(sc.cap, need);
        sc.fecap = std::max(sc.fecap, (size_t)nfe);
        PGB_CUDA(cudaMalloc(&sc.bd, sizeof(unsigned short) * sc.cap));
        PGB_CUDA(cudaMalloc(&sc.fe, sizeof(int) * sc.fecap));
        sc.dev = dev;
    }
    if (!sc.err) {
        PGB_CUDA(cudaMalloc(&sc.err, sizeof(int)));
        PGB_CUDA(cudaMallocHost(&sc.herr, sizeof(int)));
    }
}

// impl 0: mma.sync kernel; impl 1: tcgen05 kernel; impl 2: tcgen05,
// warp-specialised
static void oz_gemm_launch(int impl, int mr, int nc, int kk, const double *A, int lda, const double *B, int ldb,
                           bool tb, double *C, int ldc, cudaStream_t s)
{
    static thread_local OzScratch sc;
    if (impl == 1 || impl == 2) {
        const int ntc = (nc + UM_BN - 1) / UM_BN;
        const int nstage = (kk + UM_KC - 1) / UM_KC;
        oz_scratch(sc, (size_t)ntc * nstage * UM_BSTAGE / 2, ntc * UM_BN);
        static thread_local int attr = -1;
        if (attr != 1) {
            PGB_CUDA(cudaFuncSetAttribute(k_oz_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, UM_SMEM));
            PGB_CUDA(cudaFuncSetAttribute(k_oz_umma_ws, cudaFuncAttributeMaxDynamicSharedMemorySize, UM_SMEM));
            attr = 1;
        }
        PGB_CUDA(cudaMemsetAsync(sc.err, 0, sizeof(int), s));
        PGB_PROF(PK_GEMM, s, {
            k_oz_bimg<<<(ntc * UM_BN + 127) / 128, 128, 0, s>>>(kk, nc, B, ldb, tb ? 1 : 0, ntc, nstage, sc.bd, sc.fe);
            PGB_LAUNCHED();
            const int ntiles = (mr + UM_BM - 1) / UM_BM * ntc;
            const int grid = std::min(ntiles, device_info().sms);  // persistent: one CTA per SM
            if (impl == 2)
                k_oz_umma_ws<<<grid, WS_THREADS, UM_SMEM, s>>>(mr, nc, kk, A, lda, sc.bd, sc.fe, nstage, C, ldc,
                                                              sc.err);
            else
                k_oz_umma<<<grid, UM_THREADS, UM_SMEM, s>>>(mr, nc, kk, A, lda, sc.bd, sc.fe, nstage, C, ldc, sc.err);
            PGB_LAUNCHED();
        });
        PGB_CUDA(cudaMemcpyAsync(sc.herr, sc.err, sizeof(int), cudaMemcpyDeviceToHost, s));
        PGB_CUDA(cudaStreamSynchronize(s));
        if (*sc.herr) {
            set_error("tensor-core GEMM: an mbarrier wait ran out");
            throw WaitFailure();
        }
        return;
    }
    const int Kp = (kk + 15) / 16 * 16;
    const int ncp = (nc + OZ_BN - 1) / OZ_BN * OZ_BN;
    oz_scratch(sc, (size_t)OZ_S * ncp * Kp, ncp);
    const size_t smem = sizeof(unsigned short) * OZ_S * OZ_BN * (size_t)(Kp + 8);
    static thread_local size_t smem_set = 0;
    if (smem > 48 * 1024 && smem_set < smem) {
        PGB_CUDA(cudaFuncSetAttribute(k_oz_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        smem_set = smem;
    }
    PGB_PROF(PK_GEMM, s, {
        k_oz_bdigits<<<(ncp + 127) / 128, 128, 0, s>>>(kk, nc, B, ldb, tb ? 1 : 0, Kp, ncp, sc.bd, sc.fe);
        PGB_LAUNCHED();
        const int grid = (mr + 16 * OZ_WARPS - 1) / (16 * OZ_WARPS) * (ncp / OZ_BN);
        k_oz_gemm<<<grid, OZ_WARPS * 32, smem, s>>>(mr, nc, kk, A, lda, sc.bd, sc.fe, Kp, ncp, C, ldc);
        PGB_LAUNCHED();
    });
}

// the tcgen05 kernel of the library's restart and Ritz products
// (propack_set_gemm_impl: 1 or 2; the warp-specialised one measured 1.3x
// faster on the zipf restart products)
static std::atomic<int> g_gemm_impl{2};

bool gemm_f64_tc(int mr, int nc, int kk, const double *A, int lda, const double *B, int ldb, bool tb, double *C,
                 int ldc, cudaStream_t s)
{
    if (mr < 4096 || nc <= 0 || kk <= 0 || kk > OZ_KMAX) return false;
    oz_gemm_launch(g_gemm_impl.load(), mr, nc, kk, A, lda, B, ldb, tb, C, ldc, s);
    return true;
}

}  // namespace pgb

extern "C" int propack_set_gemm_impl(int impl)
{
    if (impl != 1 && impl != 2) return PROPACK_ERR_ARG;
    pgb::g_gemm_impl.store(impl);
    return 0;
}

// C = A op(B) with device operands through one of the tensor-core kernels
// (0: mma.sync, 1: tcgen05, 2: tcgen05 warp-specialised); all give the same
// bits.  Used by the
// tests to hold the kernels against each other and against FP64 products.
extern "C" int propack_gemm_f64_tc(int impl, int mr, int nc, int kk, const double *A, int lda, const double *B,
                                   int ldb, int tb, double *C, int ldc)
{
    using namespace pgb;
    set_error("");
    if (mr <= 0 || nc <= 0 || kk <= 0 || kk > OZ_KMAX || impl < 0 || impl > 2 || lda < mr || ldc < mr)
        return PROPACK_ERR_ARG;
    try {
        oz_gemm_launch(impl, mr, nc, kk, A, lda, B, ldb, tb != 0, C, ldc, 0);
        PGB_CUDA(cudaStreamSynchronize(0));
    } catch (const CudaFailure &) {
        return PROPACK_ERR_CUDA;
    } catch (const WaitFailure &) {
        return PROPACK_ERR_WAIT;
    }
    return 0;
}
