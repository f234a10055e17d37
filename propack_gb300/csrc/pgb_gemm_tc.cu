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
// int64 and converted to FP64 once per output: the FP64 pipe (two lanes per
// clock per SM) does ~3 operations per output instead of K FMAs.
//
// The digits of A are produced in registers from the FP64 bits with integer
// operations, straight into mma.sync fragments (m16n8k16, row.col); the
// digits of B come from a small pre-pass and are staged in shared memory.
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
            long long V = 0;
#pragma unroll
            for (int g = 0; g < OZ_S; g++) V = V * 128 + (long long)__float2int_rn(acc[g][t][r]);
            if (row < mr && col < nc) {
                const int sc = ((r < 2) ? Ea : Eb) + Fe[col] - 14 - 7 * (OZ_S - 1);
                C[(size_t)col * ldc + row] = ldexp((double)V, sc);
            }
        }
}

// scratch for the digits of B (grown on demand, per host thread)
struct OzScratch {
    unsigned short *bd = nullptr;
    int *fe = nullptr;
    size_t cap = 0;
    int dev = -1;
    ~OzScratch()
    {
        if (bd) cudaFree(bd);
        if (fe) cudaFree(fe);
    }
};

bool gemm_f64_tc(int mr, int nc, int kk, const double *A, int lda, const double *B, int ldb, bool tb, double *C,
                 int ldc, cudaStream_t s)
{
    if (mr < 4096 || nc <= 0 || kk <= 0 || kk > OZ_KMAX) return false;
    const int Kp = (kk + 15) / 16 * 16;
    const int ncp = (nc + OZ_BN - 1) / OZ_BN * OZ_BN;
    static thread_local OzScratch sc;
    int dev = 0;
    PGB_CUDA(cudaGetDevice(&dev));
    const size_t need = (size_t)OZ_S * ncp * Kp;
    if (sc.cap < need || sc.dev != dev) {
        if (sc.bd) { PGB_CUDA(cudaStreamSynchronize(s)); cudaFree(sc.bd); cudaFree(sc.fe); }
        PGB_CUDA(cudaMalloc(&sc.bd, sizeof(unsigned short) * need));
        PGB_CUDA(cudaMalloc(&sc.fe, sizeof(int) * (size_t)ncp));
        sc.cap = need;
        sc.dev = dev;
    }
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
    return true;
}

}  // namespace pgb
