// pgb_operator.cu -- the device-resident sparse operator A = S + L diag(w) R'
// (the library's APROD): upload, device-side transpose, CSR-adaptive row
// blocking, and the plain (unfused) application used by the random start
// vector (dgetu0.F:71) and by the APROD-compatible C entry point.
#include <algorithm>
#include <cstring>
#include <map>
#include <type_traits>
#include <atomic>
#include <mutex>
#include <vector>

#include "../../include/propack_gb300.h"
#include "pgb.cuh"
#include "pgb_spmv.cuh"

namespace pgb {

thread_local int64_t g_launches = 0;

// ------------------------------------------------------- event profiling
thread_local int g_prof_on = 0;
struct ProfRec {
    int kind;
    cudaEvent_t a, b;
};
static thread_local std::vector<ProfRec> g_prof_open;
static thread_local std::vector<cudaEvent_t> g_prof_pool;
static thread_local double g_prof_ms[PK_N];
static thread_local int64_t g_prof_cnt[PK_N];

static cudaEvent_t prof_event()
{
    if (!g_prof_pool.empty()) {
        cudaEvent_t e = g_prof_pool.back();
        g_prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}
void prof_mark(int kind, cudaStream_t s, bool begin)
{
    if (begin) {
        ProfRec r;
        r.kind = kind;
        r.a = prof_event();
        r.b = nullptr;
        cudaEventRecord(r.a, s);
        g_prof_open.push_back(r);
    } else if (!g_prof_open.empty()) {
        ProfRec &r = g_prof_open.back();
        r.b = prof_event();
        cudaEventRecord(r.b, s);
    }
}
void prof_collect()
{
    for (ProfRec &r : g_prof_open) {
        if (!r.b) continue;
        cudaEventSynchronize(r.b);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            g_prof_ms[r.kind] += ms;
            g_prof_cnt[r.kind] += 1;
        }
        g_prof_pool.push_back(r.a);
        g_prof_pool.push_back(r.b);
    }
    g_prof_open.clear();
}
void prof_reset()
{
    for (int i = 0; i < PK_N; i++) { g_prof_ms[i] = 0.0; g_prof_cnt[i] = 0; }
}
void prof_get(double *ms, int64_t *cnt, int n)
{
    for (int i = 0; i < n && i < PK_N; i++) { ms[i] = g_prof_ms[i]; cnt[i] = g_prof_cnt[i]; }
}
static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }
const char *last_error() { return g_err.c_str(); }

const Dev &device_info()
{
    static thread_local Dev d;
    static thread_local int cached = -1;
    int cur = 0;
    PGB_CUDA(cudaGetDevice(&cur));
    if (cached != cur) {
        cudaDeviceProp p;
        PGB_CUDA(cudaGetDeviceProperties(&p, cur));
        d.device = cur;
        d.sms = p.multiProcessorCount;
        d.nb = d.sms * 4;
        cached = cur;
    }
    return d;
}

// ------------------------------------------------------ memory pool
cudaMemPool_t lib_pool()
{
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    int dev = 0;
    PGB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    auto it = pools.find(dev);
    if (it != pools.end()) return it->second;
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool;
    PGB_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = UINT64_MAX;
    PGB_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    pools[dev] = pool;
    return pool;
}

void *pool_alloc(size_t bytes, cudaStream_t s)
{
    void *p = nullptr;
    PGB_CUDA(cudaMallocFromPoolAsync(&p, std::max<size_t>(bytes, 16), lib_pool(), s));
    return p;
}

// ------------------------------------------------------------ scans
// Exclusive prefix sum of n int counts into out[0..n] (out[n] = total).
__global__ void k_scan_blocks(const int *in, int n, int *bsum)
{
    __shared__ int sh[1024];
    const int base = blockIdx.x * 4096;
    int s = 0;
    for (int q = 0; q < 4; q++) {
        const int i = base + q * 1024 + threadIdx.x;
        s += (i < n) ? in[i] : 0;
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 512; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = sh[0];
}
__global__ void k_scan_sums(int *bsum, int nblk, int *total_out)
{
    // single CTA, sequential over chunks of 1024 with a running carry
    __shared__ int sh[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int c0 = 0; c0 < nblk; c0 += 1024) {
        const int i = c0 + threadIdx.x;
        const int v = (i < nblk) ? bsum[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            const int t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nblk) bsum[i] = carry + sh[threadIdx.x] - v;  // exclusive
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total_out = carry;
}
__global__ void k_scan_final(const int *in, int n, const int *boff, int *out)
{
    __shared__ int sh[1024];
    const int base = blockIdx.x * 4096;
    int v[4], s = 0;
    for (int q = 0; q < 4; q++) {
        const int i = base + threadIdx.x * 4 + q;
        v[q] = (i < n) ? in[i] : 0;
        s += v[q];
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int t = (threadIdx.x >= o) ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    int run = boff[blockIdx.x] + sh[threadIdx.x] - s;
    for (int q = 0; q < 4; q++) {
        const int i = base + threadIdx.x * 4 + q;
        if (i < n) out[i] = run;
        run += v[q];
    }
}
// out has n+1 entries; returns the total on the host.
int scan_excl(const int *in, int *out, int n, cudaStream_t s)
{
    const int nblk = std::max(1, (n + 4095) / 4096);
    int *bsum = nullptr;
    bsum = static_cast<decltype(bsum)>(pool_alloc(sizeof(int) * (nblk + 1), s));
    k_scan_blocks<<<nblk, 1024, 0, s>>>(in, n, bsum);
    PGB_LAUNCHED();
    k_scan_sums<<<1, 1024, 0, s>>>(bsum, nblk, out + n);
    PGB_LAUNCHED();
    k_scan_final<<<nblk, 1024, 0, s>>>(in, n, bsum, out);
    PGB_LAUNCHED();
    int total = 0;
    PGB_CUDA(cudaMemcpyAsync(&total, out + n, sizeof(int), cudaMemcpyDeviceToHost, s));
    pool_free(bsum, s);
    PGB_CUDA(cudaStreamSynchronize(s));
    return total;
}

// ------------------------------------------------------ row blocks
__global__ void k_blk_flags(const int *ptr, int rows, int half, int *flag)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        int f = (r == 0) || (r % ROWS_W == 0);
        const int len = ptr[r + 1] - ptr[r];
        if (r > 0) {
            const int lenp = ptr[r] - ptr[r - 1];
            if (ptr[r] / half != ptr[r - 1] / half) f = 1;
            if (lenp > half) f = 1;
        }
        if (len > half) f = 1;
        flag[r] = f;
    }
}
__global__ void k_blk_emit(const int *flag, const int *pos, int rows, int *blk)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
        if (flag[r]) blk[pos[r]] = r;
    if (blockIdx.x == 0 && threadIdx.x == 0) blk[pos[rows]] = rows;
}
// chunked schedule: C = max(1, ceil(E / 32)) units of 32 entries per tile
__global__ void k_chunk_count(const int *ptr, int rows, int *cnt)
{
    const int ntiles = (rows + 31) / 32;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
        const int e = ptr[min(32 * t + 32, rows)] - ptr[32 * t];
        cnt[t] = max(1, (e + 31) / 32);
    }
}
// entry p of tile t goes to unit tbase[t] + p % C, lane p / C.  One warp per
// tile: its lanes read the tile's entries, which are contiguous, with
// coalesced loads.
__global__ void k_chunk_scatter(const int *__restrict__ ptr, const int *__restrict__ idx,
                                const double *__restrict__ val, const float *__restrict__ valf, int rows,
                                const int *__restrict__ tbase, int *__restrict__ cidx, double *__restrict__ cval,
                                float *__restrict__ cvalf)
{
    const int lane = threadIdx.x & 31, ntiles = (rows + 31) / 32;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < ntiles; t += nw) {
        const int eb = ptr[32 * t], ee = ptr[min(32 * t + 32, rows)], t0 = tbase[t], C = tbase[t + 1] - t0;
#pragma unroll 4
        for (int p = lane; p < ee - eb; p += 32) {
            const int e = eb + p;
            const size_t pos = ((size_t)t0 + p % C) * 32 + p / C;
            cidx[pos] = idx[e];
            cval[pos] = val[e];
            cvalf[pos] = valf[e];
        }
    }
}

// the same for complex values (native complex operators)
__global__ void k_chunk_scatter_z(const int *__restrict__ ptr, const int *__restrict__ idx,
                                  const double2 *__restrict__ val, int rows, const int *__restrict__ tbase,
                                  int *__restrict__ cidx, double2 *__restrict__ cval)
{
    const int lane = threadIdx.x & 31, ntiles = (rows + 31) / 32;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < ntiles; t += nw) {
        const int eb = ptr[32 * t], ee = ptr[min(32 * t + 32, rows)], t0 = tbase[t], C = tbase[t + 1] - t0;
#pragma unroll 4
        for (int p = lane; p < ee - eb; p += 32) {
            const int e = eb + p;
            const size_t pos = ((size_t)t0 + p % C) * 32 + p / C;
            cidx[pos] = idx[e];
            cval[pos] = val[e];
        }
    }
}

// the run-interleaved copy of the matrix for the chunked schedule (after
// its FP32 values; complex: from its complex values)
static void build_chunks(Csr &A, cudaStream_t s)
{
    if (A.rows == 0 || A.cidx) return;
    const int ntiles = (A.rows + 31) / 32;
    int *cnt = nullptr;
    cnt = static_cast<decltype(cnt)>(pool_alloc(sizeof(int) * (ntiles + 1), s));
    A.tbase = (int *)pool_alloc(sizeof(int) * (ntiles + 1), s);
    const int g = std::min(4096, std::max(1, (ntiles + 255) / 256));
    k_chunk_count<<<g, 256, 0, s>>>(A.ptr, A.rows, cnt);
    PGB_LAUNCHED();
    const size_t units = (size_t)scan_excl(cnt, A.tbase, ntiles, s);
    pool_free(cnt, s);
    const size_t len = units * 32;
    const int gr = std::min(4096, std::max(1, (ntiles + 7) / 8));  // a warp per 32-row tile
    A.cidx = (int *)pool_alloc(sizeof(int) * len, s);
    PGB_CUDA(cudaMemsetAsync(A.cidx, 0, sizeof(int) * len, s));
    if (A.zval) {
        A.czval = (double2 *)pool_alloc(sizeof(double2) * len, s);
        PGB_CUDA(cudaMemsetAsync(A.czval, 0, sizeof(double2) * len, s));
        k_chunk_scatter_z<<<gr, 256, 0, s>>>(A.ptr, A.idx, A.zval, A.rows, A.tbase, A.cidx, A.czval);
        PGB_LAUNCHED();
        return;
    }
    A.cval = (double *)pool_alloc(sizeof(double) * len, s);
    A.cvalf = (float *)pool_alloc(sizeof(float) * len, s);
    PGB_CUDA(cudaMemsetAsync(A.cval, 0, sizeof(double) * len, s));
    PGB_CUDA(cudaMemsetAsync(A.cvalf, 0, sizeof(float) * len, s));
    k_chunk_scatter<<<gr, 256, 0, s>>>(A.ptr, A.idx, A.val, A.valf, A.rows, A.tbase, A.cidx, A.cval, A.cvalf);
    PGB_LAUNCHED();
}

static void free_chunks(Csr &A)
{
    pool_free(A.tbase, 0); pool_free(A.cidx, 0); pool_free(A.cval, 0); pool_free(A.cvalf, 0); pool_free(A.czval, 0);
    A.tbase = A.cidx = nullptr;
    A.cval = nullptr;
    A.cvalf = nullptr;
    A.czval = nullptr;
}

static void build_blocks(Csr &A, cudaStream_t s)
{
    int *flag = nullptr, *pos = nullptr;
    const int rows = A.rows;
    A.short_rows = 0;  // the schedule is chosen after the FP32 values exist (choose_schedule)
    flag = static_cast<decltype(flag)>(pool_alloc(sizeof(int) * (rows + 1), s));
    pos = static_cast<decltype(pos)>(pool_alloc(sizeof(int) * (rows + 1), s));
    const int g = std::min(4096, std::max(1, (rows + 255) / 256));
    if (rows > 0) {
        k_blk_flags<<<g, 256, 0, s>>>(A.ptr, rows, NNZ_W / 2, flag);
        PGB_LAUNCHED();
    }
    A.nblk = scan_excl(flag, pos, rows, s);
    A.blk = (int *)pool_alloc(sizeof(int) * (A.nblk + 1), s);
    k_blk_emit<<<g, 256, 0, s>>>(flag, pos, rows, A.blk);
    PGB_LAUNCHED();
    pool_free(flag, s);
    pool_free(pos, s);
}

// -------------------------------------------------------- transpose
// T = [A' | X] where X (A.cols x xcols) contributes extra entries appended
// to every row of A' with column index xoff + col.  Entries of a row of
// A' come out in increasing original position, i.e. increasing row of A,
// so the transposed SpMV sums in a fixed order.
__global__ void k_count_cols(const int *idx, int64_t nnz, int *cnt)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[idx[e]], 1);
}
__global__ void k_add_extra(int *tot, const int *cnt, const int *xptr, int cols)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x)
        tot[c] = cnt[c] + (xptr ? (xptr[c + 1] - xptr[c]) : 0);
}
// One warp per 32-row tile: the lanes read the tile's entries (contiguous)
// with coalesced loads and find each entry's row among the tile's 33 row
// starts, kept in shared memory.  The order of the atomic slots is
// arbitrary; the keys (entry, row) are sorted per column afterwards.
// Each lane takes SCATTER_BATCH entries at a time: their index loads, then
// their atomics, then their key stores, so that the round trips of a batch
// overlap.
constexpr int SCATTER_BATCH = 4;
__global__ void __launch_bounds__(256) k_scatter(const int *__restrict__ ptr, const int *__restrict__ idx, int rows,
                                                 const int *__restrict__ optr, int *__restrict__ fill,
                                                 unsigned long long *__restrict__ key)
{
    __shared__ int rbs[8][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, ntiles = (rows + 31) / 32;
    int *rb = rbs[w];
    const int nw = gridDim.x * 8;
    for (int t = blockIdx.x * 8 + w; t < ntiles; t += nw) {
        rb[lane] = ptr[min(32 * t + lane, rows)];
        if (lane == 0) rb[32] = ptr[min(32 * t + 32, rows)];
        __syncwarp();
        const int eb = rb[0], ee = rb[32];
        for (int e0 = eb + lane; e0 < ee; e0 += 32 * SCATTER_BATCH) {
            int c[SCATTER_BATCH], p[SCATTER_BATCH];
#pragma unroll
            for (int u = 0; u < SCATTER_BATCH; u++) {
                const int e = e0 + 32 * u;
                c[u] = e < ee ? idx[e] : 0;
            }
#pragma unroll
            for (int u = 0; u < SCATTER_BATCH; u++)
                p[u] = e0 + 32 * u < ee ? optr[c[u]] + atomicAdd(&fill[c[u]], 1) : 0;
#pragma unroll
            for (int u = 0; u < SCATTER_BATCH; u++) {
                const int e = e0 + 32 * u;
                if (e >= ee) break;
                // the last row of the tile that starts at or before e
                int k = 0;
#pragma unroll
                for (int st = 16; st > 0; st >>= 1)
                    if (rb[k + st] <= e) k += st;
                key[p[u]] = ((unsigned long long)(unsigned)e << 32) | (unsigned)(32 * t + k);
            }
        }
        __syncwarp();
    }
}
// segments of at most SEG_SMALL keys (most columns of a sparse matrix): one
// thread per segment, insertion sort in registers/local memory.  The keys
// are distinct, so every sort gives the same order.
constexpr int SEG_SMALL = 32;
__global__ void k_segsort_small(unsigned long long *key, const int *optr, const int *cnt, int cols)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x) {
        const int len = cnt[c], off = optr[c];
        if (len <= 1 || len > SEG_SMALL) continue;
        if (len <= 8) {
            // the common case, in registers: an odd-even transposition
            // network over eight keys padded with the largest key
            unsigned long long r[8];
#pragma unroll
            for (int i = 0; i < 8; i++) r[i] = i < len ? key[off + i] : ~0ull;
#pragma unroll
            for (int round = 0; round < 8; round++)
#pragma unroll
                for (int i = round & 1; i + 1 < 8; i += 2) {
                    const unsigned long long a = r[i], b = r[i + 1];
                    r[i] = a < b ? a : b;
                    r[i + 1] = a < b ? b : a;
                }
#pragma unroll
            for (int i = 0; i < 8; i++)
                if (i < len) key[off + i] = r[i];
            continue;
        }
        unsigned long long v[SEG_SMALL];
        for (int i = 0; i < len; i++) v[i] = key[off + i];
        for (int i = 1; i < len; i++) {
            const unsigned long long x = v[i];
            int j = i - 1;
            while (j >= 0 && v[j] > x) {
                v[j + 1] = v[j];
                j--;
            }
            v[j + 1] = x;
        }
        for (int i = 0; i < len; i++) key[off + i] = v[i];
    }
}
// one warp per segment of SEG_SMALL+1 .. 1024 keys: bitonic sort in shared
// memory; longer segments are listed for k_segsort_long.
__global__ void k_segsort_warp(unsigned long long *key, const int *optr, const int *cnt, int cols,
                               int *longlist, int *nlong)
{
    __shared__ unsigned long long sh[4][1024];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned long long *s = sh[w];
    for (int c = blockIdx.x * 4 + w; c < cols; c += gridDim.x * 4) {
        const int len = cnt[c], off = optr[c];
        if (len <= SEG_SMALL) continue;
        if (len > 1024) {
            if (lane == 0) longlist[atomicAdd(nlong, 1)] = c;
            continue;
        }
        int P = 2;
        while (P < len) P <<= 1;
        for (int i = lane; i < P; i += 32) s[i] = (i < len) ? key[off + i] : ~0ull;
        __syncwarp();
        for (int k = 2; k <= P; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = lane; i < P; i += 32) {
                    const int ixj = i ^ j;
                    if (ixj > i) {
                        const unsigned long long a = s[i], b = s[ixj];
                        const bool up = ((i & k) == 0);
                        if ((a > b) == up) { s[i] = b; s[ixj] = a; }
                    }
                }
                __syncwarp();
            }
        }
        for (int i = lane; i < len; i += 32) key[off + i] = s[i];
        __syncwarp();
    }
}
// one CTA per long segment: bitonic sort in a padded global scratch area
__global__ void k_segsort_long(unsigned long long *key, const int *optr, const int *cnt, const int *list,
                               const int64_t *soff, unsigned long long *scratch)
{
    const int c = list[blockIdx.x];
    const int len = cnt[c], off = optr[c];
    unsigned long long *s = scratch + soff[blockIdx.x];
    int P = 2;
    while (P < len) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) s[i] = (i < len) ? key[off + i] : ~0ull;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const unsigned long long a = s[i], b = s[ixj];
                    const bool up = ((i & k) == 0);
                    if ((a > b) == up) { s[i] = b; s[ixj] = a; }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < len; i += blockDim.x) key[off + i] = s[i];
}
// the value of A' (real) or of A^H (complex: conjugated)
__device__ __forceinline__ double adj_value(double v) { return v; }
__device__ __forceinline__ double2 adj_value(double2 v) { return make_double2(v.x, -v.y); }
template <typename V>
__global__ void k_finish_t(const unsigned long long *key, const int *optr, const int *cnt, int cols,
                           const V *val, const int *xptr, const int *xidx, const V *xval, int xoff,
                           int *oidx, V *oval)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < cols; c += gridDim.x * blockDim.x) {
        const int off = optr[c], len = cnt[c];
        for (int q = 0; q < len; q++) {
            const unsigned long long k = key[off + q];
            oidx[off + q] = (int)(k & 0xffffffffull);
            oval[off + q] = adj_value(val[(int)(k >> 32)]);
        }
        if (xptr) {
            int p = off + len;
            for (int e = xptr[c]; e < xptr[c + 1]; e++, p++) {
                oidx[p] = xoff + xidx[e];
                oval[p] = xval[e];
            }
        }
    }
}

// without appended X entries every key slot p holds an entry of A: one
// thread per slot (coalesced index and value writes)
// (four slots per thread and round, so that four value gathers are in
// flight)
template <typename V>
__global__ void k_finish_t_flat(const unsigned long long *__restrict__ key, int64_t total, const V *__restrict__ val,
                                int *__restrict__ oidx, V *__restrict__ oval)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t p0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p0 < total; p0 += 4 * stride) {
        unsigned long long k[4];
        V v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) k[u] = p0 + u * stride < total ? key[p0 + u * stride] : 0ull;
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (p0 + u * stride < total) v[u] = val[(int)(k[u] >> 32)];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int64_t p = p0 + u * stride;
            if (p >= total) break;
            oidx[p] = (int)(k[u] & 0xffffffffull);
            oval[p] = adj_value(v[u]);
        }
    }
}

// A: rows x cols device CSR (ptr/idx/val); X optional (cols rows).  V =
// double2: a complex A, T = A^H (X must be absent), values into T.zval.
template <typename V>
static void transpose_into(Csr &T, const int *ptr, const int *idx, const V *val, int rows, int cols,
                           int64_t nnz, const int *xptr, const int *xidx, const V *xval, int xoff, int xcols,
                           cudaStream_t s)
{
    constexpr bool Z = std::is_same<V, double2>::value;
    int *cnt = nullptr, *tot = nullptr, *fill = nullptr, *longlist = nullptr, *nlong = nullptr;
    unsigned long long *key = nullptr;
    cnt = static_cast<decltype(cnt)>(pool_alloc(sizeof(int) * (cols + 1), s));
    tot = static_cast<decltype(tot)>(pool_alloc(sizeof(int) * (cols + 1), s));
    fill = static_cast<decltype(fill)>(pool_alloc(sizeof(int) * (cols + 1), s));
    longlist = static_cast<decltype(longlist)>(pool_alloc(sizeof(int) * (cols + 1), s));
    nlong = static_cast<decltype(nlong)>(pool_alloc(sizeof(int), s));
    PGB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (cols + 1), s));
    PGB_CUDA(cudaMemsetAsync(fill, 0, sizeof(int) * (cols + 1), s));
    PGB_CUDA(cudaMemsetAsync(nlong, 0, sizeof(int), s));
    const int g = 4096;
    if (nnz > 0) { k_count_cols<<<g, 256, 0, s>>>(idx, nnz, cnt); PGB_LAUNCHED(); }
    if (cols > 0) { k_add_extra<<<g, 256, 0, s>>>(tot, cnt, xptr, cols); PGB_LAUNCHED(); }
    T.rows = cols;
    T.cols = rows + xcols;
    T.ncol0 = rows;
    T.ptr = (int *)pool_alloc(sizeof(int) * (cols + 1), s);
    const int total = scan_excl(tot, T.ptr, cols, s);
    T.nnz = total;
    T.idx = (int *)pool_alloc(sizeof(int) * std::max(total, 1), s);
    V *tval = (V *)pool_alloc(sizeof(V) * std::max(total, 1), s);
    if constexpr (Z) T.zval = tval;
    else T.val = tval;
    // the sort keys live at the output positions of row c of A', whose
    // offsets T.ptr include the appended X entries: size them by `total`,
    // not by nnz(A)
    key = static_cast<decltype(key)>(pool_alloc(sizeof(unsigned long long) * std::max(total, 1), s));
    // the scan wrote T.ptr; optr == T.ptr, the A' part of row c is [ptr[c], ptr[c]+cnt[c])
    if (rows > 0 && nnz > 0) {
        const int gt = std::min(4096, std::max(1, ((rows + 31) / 32 + 7) / 8));  // a warp per 32-row tile
        k_scatter<<<gt, 256, 0, s>>>(ptr, idx, rows, T.ptr, fill, key);
        PGB_LAUNCHED();
    }
    if (cols > 0) {
        k_segsort_small<<<g, 256, 0, s>>>(key, T.ptr, cnt, cols);
        PGB_LAUNCHED();
        k_segsort_warp<<<g, 128, 0, s>>>(key, T.ptr, cnt, cols, longlist, nlong);
        PGB_LAUNCHED();
    }
    int hlong = 0;
    PGB_CUDA(cudaMemcpyAsync(&hlong, nlong, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGB_CUDA(cudaStreamSynchronize(s));
    if (hlong > 0) {
        std::vector<int> hl(hlong), hc(hlong);
        PGB_CUDA(cudaMemcpy(hl.data(), longlist, sizeof(int) * hlong, cudaMemcpyDeviceToHost));
        std::sort(hl.begin(), hl.end());
        std::vector<int64_t> soff(hlong + 1, 0);
        for (int q = 0; q < hlong; q++) {
            int len = 0;
            PGB_CUDA(cudaMemcpy(&len, cnt + hl[q], sizeof(int), cudaMemcpyDeviceToHost));
            int64_t P = 2;
            while (P < len) P <<= 1;
            soff[q + 1] = soff[q] + P;
        }
        int *dl = nullptr;
        int64_t *doff = nullptr;
        unsigned long long *scr = nullptr;
        PGB_CUDA(cudaMalloc(&dl, sizeof(int) * hlong));
        PGB_CUDA(cudaMalloc(&doff, sizeof(int64_t) * (hlong + 1)));
        PGB_CUDA(cudaMalloc(&scr, sizeof(unsigned long long) * soff[hlong]));
        PGB_CUDA(cudaMemcpy(dl, hl.data(), sizeof(int) * hlong, cudaMemcpyHostToDevice));
        PGB_CUDA(cudaMemcpy(doff, soff.data(), sizeof(int64_t) * (hlong + 1), cudaMemcpyHostToDevice));
        k_segsort_long<<<hlong, 1024, 0, s>>>(key, T.ptr, cnt, dl, doff, scr);
        PGB_LAUNCHED();
        PGB_CUDA(cudaStreamSynchronize(s));
        PGB_CUDA(cudaFree(dl));
        PGB_CUDA(cudaFree(doff));
        PGB_CUDA(cudaFree(scr));
    }
    if (cols > 0 && !xptr) {
        if (total > 0) {
            k_finish_t_flat<V><<<g, 256, 0, s>>>(key, total, val, T.idx, tval);
            PGB_LAUNCHED();
        }
    } else if (cols > 0) {
        k_finish_t<V><<<g, 256, 0, s>>>(key, T.ptr, cnt, cols, val, xptr, xidx, xval, rows, T.idx, tval);
        PGB_LAUNCHED();
    }
    pool_free(cnt, s);
    pool_free(tot, s);
    pool_free(fill, s);
    pool_free(longlist, s);
    pool_free(nlong, s);
    pool_free(key, s);
    (void)xoff;
}

// fwd = [S | L]: row i holds S's row then L's row (columns n + c)
__global__ void k_count_merge(const int *sp, const int *lp, int rows, int *tot)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x)
        tot[i] = (sp[i + 1] - sp[i]) + (lp ? (lp[i + 1] - lp[i]) : 0);
}
__global__ void k_merge_rows(const int *sp, const int *si, const double *sv, const int *lp, const int *li,
                             const double *lv, int rows, int loff, const int *optr, int *oi, double *ov)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x) {
        int p = optr[i];
        for (int e = sp[i]; e < sp[i + 1]; e++, p++) { oi[p] = si[e]; ov[p] = sv[e]; }
        if (lp)
            for (int e = lp[i]; e < lp[i + 1]; e++, p++) { oi[p] = loff + li[e]; ov[p] = lv[e]; }
    }
}
__global__ void k_to_float(const double *a, float *b, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// ------------------------------------------------------ application
// z[c] = w[c] * sum(thin row c . x), split into segments of NNZ_PB.  The
// low-rank coefficients are always formed in FP64.
template <typename T>
__global__ void __launch_bounds__(BS) k_thin(Csr Th, const T *__restrict__ x, const double *w, double *zpart,
                                             double *z, unsigned int *ticket)
{
    __shared__ double sred[32];
    const int nseg = Th.segs;
    for (int t = blockIdx.x; t < Th.rows * nseg; t += gridDim.x) {
        const int c = t / nseg, sg = t % nseg;
        const int a = Th.ptr[c] + sg * NNZ_PB;
        const int b = min(Th.ptr[c + 1], a + NNZ_PB);
        double acc = 0.0;
        for (int e = a + threadIdx.x; e < b; e += BS) acc += Th.val[e] * (double)x[Th.idx[e]];
        acc = block_sum<BS>(acc, sred);
        if (threadIdx.x == 0) zpart[t] = acc;
    }
    if (last_cta(ticket)) {
        for (int c = threadIdx.x; c < Th.rows; c += BS) {
            double s = 0.0;
            for (int sg = 0; sg < nseg; sg++) s += zpart[c * nseg + sg];
            z[c] = w[c] * s;
        }
    }
}

template <typename T>
__device__ __forceinline__ const T *plain_vals(const Csr &A);
template <>
__device__ __forceinline__ const double *plain_vals<double>(const Csr &A) { return A.val; }
template <>
__device__ __forceinline__ const float *plain_vals<float>(const Csr &A) { return A.valf; }

// y = A x (A = fwd or adj) with x already carrying z for the tail columns
template <typename T>
__global__ void __launch_bounds__(BS) k_spmv_plain(Csr A, const T *__restrict__ x, const double *__restrict__ z,
                                                   T *__restrict__ y)
{
    __shared__ SpmvStage<T, T> st[SPMV_WARPS];
    __shared__ ChunkStage<T> cst[SPMV_WARPS];
    const int n0 = A.ncol0;
    auto xl = [&](int c) -> T { return c < n0 ? __ldg(x + c) : (T)z[c - n0]; };
    auto pre = [&](int r) -> double { return 0.0; };
    auto epi = [&](int r, double acc, double) { y[r] = (T)acc; };
    csr_spmv<T, T>(A, plain_vals<T>(A), xl, pre, epi, st, cst);
}

// one wave of CTAs at the kernel's occupancy
// (cached per host thread for the current device; recomputed when the
// thread moves to another device)
template <typename T>
static int spmv_plain_grid()
{
    static thread_local int g = 0, dev = -1;
    const Dev &d = device_info();
    if (g == 0 || dev != d.device) {
        int per = 0;
        PGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_spmv_plain<T>, BS, 0));
        g = std::max(1, per) * d.sms;
        dev = d.device;
    }
    return g;
}

template <typename T>
void op_thin(const Operator &op, bool trans, const T *x, cudaStream_t s)
{
    if (op.r <= 0) return;
    const Csr &Th = trans ? op.thin_l : op.thin_r;
    const int nt = std::max(1, Th.rows * Th.segs);
    k_thin<T><<<std::min(nt, device_info().nb), BS, 0, s>>>(Th, x, op.w, op.zpart, op.zbuf, op.zticket);
    PGB_LAUNCHED();
}

// y = A x with a caller-supplied z (the low-rank coefficients); no scratch
void op_spmv_plain_launch(const Csr &A, const double *x, const double *z, double *y, cudaStream_t s)
{
    k_spmv_plain<double><<<spmv_plain_grid<double>(), BS, 0, s>>>(A, x, z, y);
    PGB_LAUNCHED();
}

// ------------------------------------------------- schedule selection
// propack_set_spmv_schedule: 0 the row-length rule (default), 1 chunked,
// 2 staged, 3 timed choice
static std::atomic<int> g_sched{0};
constexpr int CHUNK_RULE_MEAN = 128;  // the rule: chunked below this mean row length
constexpr int CHUNK_MEAN_MAX = 512;   // the timed choice tries the chunked schedule below this mean row length

// mean device ms of one plain product with the matrix's current schedule
static float time_spmv(const Csr &A, const double *x, const double *z, double *y, cudaStream_t s)
{
    cudaEvent_t e0, e1;
    PGB_CUDA(cudaEventCreate(&e0));
    PGB_CUDA(cudaEventCreate(&e1));
    op_spmv_plain_launch(A, x, z, y, s);
    PGB_CUDA(cudaEventRecord(e0, s));
    for (int i = 0; i < 3; i++) op_spmv_plain_launch(A, x, z, y, s);
    PGB_CUDA(cudaEventRecord(e1, s));
    PGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    PGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / 3.f;
}

// Sets A.short_rows (1: chunked, 0: staged).  The default is a rule on the
// mean row length (chunked below CHUNK_RULE_MEAN, where it measured faster
// on every workload tried: 7.7, 20.6 and ~83 nonzeros per row), so that a given
// matrix always gets the same schedule and the same summation order.  The
// timed choice (mode 3) builds the chunked copy, runs both schedules on the
// device and keeps the chunked one when it wins; it starts from the rule
// and switches only when the other schedule is more than 5 % faster, but a
// near-tie can still go either way between builds, and with it the last
// bits of every product.
static void choose_schedule(Csr &A, const double *z, cudaStream_t s)
{
    const int mode = g_sched.load();
    const bool rule = A.rows > 0 && A.nnz < (int64_t)CHUNK_RULE_MEAN * A.rows;
    A.short_rows = 0;
    if (A.rows == 0 || mode == 2) return;
    if (mode == 1 || (mode == 0 && rule)) {
        build_chunks(A, s);
        A.short_rows = 1;
        return;
    }
    if (mode == 0) return;
    if (A.nnz >= (int64_t)CHUNK_MEAN_MAX * A.rows) return;
    build_chunks(A, s);
    double *x = nullptr, *y = nullptr;
    x = static_cast<decltype(x)>(pool_alloc(sizeof(double) * std::max(A.ncol0, 1), s));
    y = static_cast<decltype(y)>(pool_alloc(sizeof(double) * A.rows, s));
    PGB_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * std::max(A.ncol0, 1), s));
    A.short_rows = 1;
    const float tc = time_spmv(A, x, z, y, s);
    A.short_rows = 0;
    const float ts = time_spmv(A, x, z, y, s);
    pool_free(x, s);
    pool_free(y, s);
    const bool chunked = rule ? !(ts < 0.95f * tc) : (tc < 0.95f * ts);
    A.short_rows = chunked ? 1 : 0;
    A.tuned_ms[0] = tc;
    A.tuned_ms[1] = ts;
    if (!chunked) {
        PGB_CUDA(cudaStreamSynchronize(s));
        free_chunks(A);
    }
}

template <typename T>
void op_apply(const Operator &op, bool trans, const T *x, T *y, cudaStream_t s)
{
    op_thin<T>(op, trans, x, s);
    const Csr &A = trans ? op.adj : op.fwd;
    k_spmv_plain<T><<<spmv_plain_grid<T>(), BS, 0, s>>>(A, x, op.zbuf, y);
    PGB_LAUNCHED();
}
// y = A x for one side of a native complex operator (chunked schedule,
// complex accumulation)
__global__ void __launch_bounds__(BS) k_zspmv_plain(Csr A, const double2 *__restrict__ x, double2 *__restrict__ y)
{
    __shared__ ChunkStage<double2> cst[SPMV_WARPS];
    auto xl = [&](int c) -> double2 { return x[c]; };
    auto pre = [&](int) -> double { return 0.0; };
    auto epi = [&](int r, double2 acc, double) { y[r] = acc; };
    csr_rows_chunked<double2, double2>(A.ptr, A.tbase, A.cidx, A.czval, A.rows, xl, pre, epi, cst);
}
static int zspmv_plain_grid()
{
    static thread_local int g = 0, dev = -1;
    const Dev &d = device_info();
    if (g == 0 || dev != d.device) {
        int per = 0;
        PGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_zspmv_plain, BS, 0));
        g = std::max(1, per) * d.sms;
        dev = d.device;
    }
    return g;
}
void op_zspmv_plain_launch(const Csr &A, const double2 *x, double2 *y, cudaStream_t s)
{
    k_zspmv_plain<<<zspmv_plain_grid(), BS, 0, s>>>(A, x, y);
    PGB_LAUNCHED();
}
void op_zapply(const Operator &op, bool trans, const double2 *x, double2 *y, cudaStream_t s)
{
    if (op.cplx == 2) op_zspmv_plain_launch(trans ? op.adj : op.fwd, x, y, s);
    else op_apply<double>(op, trans, (const double *)x, (double *)y, s);
}

template void op_thin<double>(const Operator &, bool, const double *, cudaStream_t);
template void op_thin<float>(const Operator &, bool, const float *, cudaStream_t);
template void op_apply<double>(const Operator &, bool, const double *, double *, cudaStream_t);
template void op_apply<float>(const Operator &, bool, const float *, float *, cudaStream_t);

// ------------------------------------------------------- registry
static std::mutex g_reg_mu;
static std::map<int64_t, Operator *> g_reg;
static int64_t g_next_id = 1;

Operator *lookup_operator(int64_t handle)
{
    std::lock_guard<std::mutex> lk(g_reg_mu);
    auto it = g_reg.find(handle);
    return it == g_reg.end() ? nullptr : it->second;
}

static void free_csr(Csr &A)
{
    pool_free(A.ptr, 0); pool_free(A.idx, 0); pool_free(A.val, 0); pool_free(A.valf, 0); pool_free(A.blk, 0);
    pool_free(A.zval, 0);
    free_chunks(A);
    A = Csr();
}

// row pointers: int64 on the host, int32 on the device; flag |= 1 unless
// 0 = p[0] <= p[1] <= ... <= p[rows] = nnz
__global__ void k_ptr_narrow(const int64_t *p, int rows, int64_t nnz, int *out, int *flag)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= rows; i += gridDim.x * blockDim.x) {
        const int64_t v = p[i];
        out[i] = (int)v;
        const bool bad = (i == 0 && v != 0) || (i == rows && v != nnz) || (i < rows && p[i + 1] < v);
        if (bad) atomicOr(flag, 1);
    }
}
// flag |= 2 when a column index lies outside [0, limit)
__global__ void k_check_idx(const int *idx, int64_t nnz, int limit, int *flag)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
        if ((unsigned)idx[e] >= (unsigned)limit) atomicOr(flag, 2);
}

template <typename T>
static T *upload(const T *p, int64_t n, cudaStream_t s)
{
    T *d = (T *)pool_alloc(sizeof(T) * std::max<int64_t>(n, 1), s);
    if (n > 0) h2d_bytes(d, p, sizeof(T) * n, s);
    return d;
}
static int *upload_ptr(const int64_t *p, int rows, int64_t nnz, int *flag, cudaStream_t s)
{
    int64_t *d64 = upload<int64_t>(p, rows + 1, s);
    int *d = (int *)pool_alloc(sizeof(int) * (rows + 1), s);
    k_ptr_narrow<<<std::min(4096, rows / 256 + 1), 256, 0, s>>>(d64, rows, nnz, d, flag);
    PGB_LAUNCHED();
    pool_free(d64, s);
    return d;
}
static void check_idx(const int *idx, int64_t nnz, int limit, int *flag, cudaStream_t s)
{
    if (nnz <= 0) return;
    k_check_idx<<<(int)std::min<int64_t>(4096, nnz / 256 + 1), 256, 0, s>>>(idx, nnz, limit, flag);
    PGB_LAUNCHED();
}

static int create_operator(int m, int n, const int64_t *sp, const int32_t *si, const double *sv, int r,
                           const int64_t *lp, const int32_t *li, const double *lv, const int64_t *rp,
                           const int32_t *ri, const double *rv, const double *w, int64_t *handle)
{
    if (m <= 0 || n <= 0 || r < 0 || !sp || !handle) throw ArgFailure();
    const int64_t snnz = sp[m];
    const int64_t lnnz = r > 0 ? lp[m] : 0, rnnz = r > 0 ? rp[n] : 0;
    if (snnz < 0 || snnz + lnnz >= (int64_t)INT32_MAX || snnz + rnnz >= (int64_t)INT32_MAX) {
        set_error("operator has 2^31 or more nonzeros");
        throw ArgFailure();
    }
    if (r > 0 && (!lp || !li || !lv || !rp || !ri || !rv || !w)) throw ArgFailure();
    device_info();
    cudaStream_t s;
    PGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    // the arrays are checked on the device before any kernel indexes by
    // them: monotone row pointers ending at nnz, column indices in range
    int *dflag = (int *)pool_alloc(sizeof(int), s);
    PGB_CUDA(cudaMemsetAsync(dflag, 0, sizeof(int), s));
    int *dsp = upload_ptr(sp, m, snnz, dflag, s);
    int *dsi = upload<int>(si, snnz, s);
    double *dsv = upload<double>(sv, snnz, s);
    check_idx(dsi, snnz, n, dflag, s);
    int *dlp = nullptr, *dli = nullptr, *drp = nullptr, *dri = nullptr;
    double *dlv = nullptr, *drv = nullptr, *dw = nullptr;
    if (r > 0) {
        dlp = upload_ptr(lp, m, lnnz, dflag, s); dli = upload<int>(li, lnnz, s); dlv = upload<double>(lv, lnnz, s);
        drp = upload_ptr(rp, n, rnnz, dflag, s); dri = upload<int>(ri, rnnz, s); drv = upload<double>(rv, rnnz, s);
        dw = upload<double>(w, r, s);
        check_idx(dli, lnnz, r, dflag, s);
        check_idx(dri, rnnz, r, dflag, s);
    }
    int hflag = 0;
    PGB_CUDA(cudaMemcpyAsync(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGB_CUDA(cudaStreamSynchronize(s));
    pool_free(dflag, s);
    if (hflag) {
        for (void *p : {(void *)dsp, (void *)dsi, (void *)dsv, (void *)dlp, (void *)dli, (void *)dlv, (void *)drp,
                        (void *)dri, (void *)drv, (void *)dw})
            pool_free(p, s);
        PGB_CUDA(cudaStreamSynchronize(s));
        cudaStreamDestroy(s);
        set_error(hflag & 1 ? "row pointers are not monotone from 0 to nnz" : "column index out of range");
        throw ArgFailure();
    }
    Operator *op = new Operator();
    op->m = m; op->n = n; op->r = r;
    op->w = dw;
    PGB_CUDA(cudaGetDevice(&op->device));
    const int g = 4096;
    // the transposition's inputs (the uploaded S)
    const int *tsp = dsp, *tsi = dsi;
    const double *tsv = dsv;
    // fwd = [S | L]; without a low-rank term that is S itself, whose
    // uploaded arrays the operator keeps
    if (r == 0) {
        Csr &A = op->fwd;
        A.rows = m; A.cols = n; A.ncol0 = n;
        A.ptr = dsp; A.idx = dsi; A.val = dsv; A.nnz = snnz;
        dsp = nullptr; dsi = nullptr; dsv = nullptr;  // owned by the operator now
        build_blocks(A, s);
    } else {
        Csr &A = op->fwd;
        A.rows = m; A.cols = n + r; A.ncol0 = n;
        int *tot = nullptr;
        tot = static_cast<decltype(tot)>(pool_alloc(sizeof(int) * (m + 1), s));
        k_count_merge<<<g, 256, 0, s>>>(dsp, dlp, m, tot);
        PGB_LAUNCHED();
        A.ptr = (int *)pool_alloc(sizeof(int) * (m + 1), s);
        A.nnz = scan_excl(tot, A.ptr, m, s);
        A.idx = (int *)pool_alloc(sizeof(int) * std::max<int64_t>(A.nnz, 1), s);
        A.val = (double *)pool_alloc(sizeof(double) * std::max<int64_t>(A.nnz, 1), s);
        k_merge_rows<<<g, 256, 0, s>>>(dsp, dsi, dsv, dlp, dli, dlv, m, n, A.ptr, A.idx, A.val);
        PGB_LAUNCHED();
        pool_free(tot, s);
        build_blocks(A, s);
    }
    // adj = [S' | R]
    transpose_into<double>(op->adj, tsp, tsi, tsv, m, n, snnz, drp, dri, drv, m, r, s);
    build_blocks(op->adj, s);
    if (r > 0) {
        // thin_r = R' (r x n), thin_l = L' (r x m)
        transpose_into<double>(op->thin_r, drp, dri, drv, n, r, rnnz, nullptr, nullptr, nullptr, 0, 0, s);
        transpose_into<double>(op->thin_l, dlp, dli, dlv, m, r, lnnz, nullptr, nullptr, nullptr, 0, 0, s);
        for (Csr *T : {&op->thin_r, &op->thin_l}) {
            std::vector<int> hp(r + 1);
            PGB_CUDA(cudaMemcpy(hp.data(), T->ptr, sizeof(int) * (r + 1), cudaMemcpyDeviceToHost));
            int mx = 0;
            for (int c = 0; c < r; c++) mx = std::max(mx, hp[c + 1] - hp[c]);
            T->segs = std::max(1, (mx + NNZ_PB - 1) / NNZ_PB);
        }
        const int segs = std::max(op->thin_r.segs, op->thin_l.segs);
        PGB_CUDA(cudaMalloc(&op->zbuf, sizeof(double) * r));
        PGB_CUDA(cudaMalloc(&op->zpart, sizeof(double) * (size_t)r * segs));
        PGB_CUDA(cudaMemset(op->zbuf, 0, sizeof(double) * r));
    }
    PGB_CUDA(cudaMalloc(&op->zticket, sizeof(unsigned int)));
    PGB_CUDA(cudaMemset(op->zticket, 0, sizeof(unsigned int)));
    // FP32 copies of the values for the mixed-precision path
    for (Csr *A : {&op->fwd, &op->adj}) {
        A->valf = (float *)pool_alloc(sizeof(float) * std::max<int64_t>(A->nnz, 1), s);
        k_to_float<<<g, 256, 0, s>>>(A->val, A->valf, A->nnz);
        PGB_LAUNCHED();
        choose_schedule(*A, op->zbuf, s);
    }
    PGB_CUDA(cudaStreamSynchronize(s));
    for (void *p : {(void *)dsp, (void *)dsi, (void *)dsv, (void *)dlp, (void *)dli, (void *)dlv, (void *)drp,
                    (void *)dri, (void *)drv})
        pool_free(p, s);
    PGB_CUDA(cudaStreamSynchronize(s));
    PGB_CUDA(cudaStreamDestroy(s));
    {
        std::lock_guard<std::mutex> lk(g_reg_mu);
        op->id = g_next_id++;
        g_reg[op->id] = op;
    }
    *handle = op->id;
    return 0;
}

// A complex m x n CSR matrix held natively: int32 column index and
// complex*16 value per entry (20 bytes, where the real 2x2-block form reads
// 4 x 12), fwd = A and adj = A^H (the device transposition, conjugating),
// both on the chunked schedule.  Checked on the device like the real
// operator before any kernel indexes by it.
static int create_zoperator(int m, int n, const int64_t *sp, const int32_t *si, const propack_z16 *sv,
                            int64_t *handle)
{
    const int64_t nnz = sp[m];
    if (nnz < 0 || nnz >= (int64_t)INT32_MAX) {
        set_error("complex operator has 2^31 or more nonzeros");
        throw ArgFailure();
    }
    if (nnz > 0 && (!si || !sv)) throw ArgFailure();
    device_info();
    cudaStream_t s;
    PGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    int *dflag = (int *)pool_alloc(sizeof(int), s);
    PGB_CUDA(cudaMemsetAsync(dflag, 0, sizeof(int), s));
    int *dsp = upload_ptr(sp, m, nnz, dflag, s);
    int *dsi = upload<int>(si, nnz, s);
    // propack_z16 is (re, im) doubles, the layout of double2
    double2 *dsv = (double2 *)pool_alloc(sizeof(double2) * std::max<int64_t>(nnz, 1), s);
    if (nnz > 0) h2d_bytes(dsv, sv, sizeof(double2) * nnz, s);
    check_idx(dsi, nnz, n, dflag, s);
    int hflag = 0;
    PGB_CUDA(cudaMemcpyAsync(&hflag, dflag, sizeof(int), cudaMemcpyDeviceToHost, s));
    PGB_CUDA(cudaStreamSynchronize(s));
    pool_free(dflag, s);
    if (hflag) {
        pool_free(dsp, s); pool_free(dsi, s); pool_free(dsv, s);
        PGB_CUDA(cudaStreamSynchronize(s));
        cudaStreamDestroy(s);
        set_error(hflag & 1 ? "row pointers are not monotone from 0 to nnz" : "column index out of range");
        throw ArgFailure();
    }
    Operator *op = new Operator();
    op->m = m; op->n = n; op->r = 0;
    op->cplx = 2;
    PGB_CUDA(cudaGetDevice(&op->device));
    Csr &A = op->fwd;
    A.rows = m; A.cols = n; A.ncol0 = n; A.nnz = nnz;
    A.ptr = dsp; A.idx = dsi; A.zval = dsv;
    transpose_into<double2>(op->adj, dsp, dsi, dsv, m, n, nnz, nullptr, nullptr, nullptr, 0, 0, s);
    for (Csr *M : {&op->fwd, &op->adj}) {
        build_chunks(*M, s);
        M->short_rows = 1;
    }
    PGB_CUDA(cudaMalloc(&op->zticket, sizeof(unsigned int)));
    PGB_CUDA(cudaMemset(op->zticket, 0, sizeof(unsigned int)));
    PGB_CUDA(cudaStreamSynchronize(s));
    PGB_CUDA(cudaStreamDestroy(s));
    {
        std::lock_guard<std::mutex> lk(g_reg_mu);
        op->id = g_next_id++;
        g_reg[op->id] = op;
    }
    *handle = op->id;
    return 0;
}

static int destroy_operator(int64_t handle)
{
    Operator *op = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_reg_mu);
        auto it = g_reg.find(handle);
        if (it == g_reg.end()) return PROPACK_ERR_HANDLE;
        op = it->second;
        g_reg.erase(it);
    }
    cudaDeviceSynchronize();
    free_csr(op->fwd); free_csr(op->adj); free_csr(op->thin_r); free_csr(op->thin_l);
    pool_free(op->w, 0);
    cudaFree(op->zbuf); cudaFree(op->zpart); cudaFree(op->zticket);
    delete op;
    return 0;
}

int64_t handle_from_iparm(const int *iparm)
{
    if (!iparm) return 0;
    return (int64_t)((uint64_t)(uint32_t)iparm[0] | ((uint64_t)(uint32_t)iparm[1] << 32));
}

}  // namespace pgb

// ------------------------------------------------------------ C ABI
using namespace pgb;

extern "C" int propack_csr_create(int m, int n, const int64_t *s_rowptr, const int32_t *s_colidx,
                                  const double *s_val, int r, const int64_t *l_rowptr, const int32_t *l_colidx,
                                  const double *l_val, const int64_t *r_rowptr, const int32_t *r_colidx,
                                  const double *r_val, const double *w, int64_t *handle)
{
    try {
        return create_operator(m, n, s_rowptr, s_colidx, s_val, r, l_rowptr, l_colidx, l_val, r_rowptr, r_colidx,
                               r_val, w, handle);
    } catch (const CudaFailure &) {
        return PROPACK_ERR_CUDA;
    } catch (const ArgFailure &) {
        if (g_err.empty()) set_error("invalid argument to propack_csr_create");
        return PROPACK_ERR_ARG;
    }
}

extern "C" int propack_csr_destroy(int64_t handle) { return destroy_operator(handle); }

// Row 2i of the real form holds (2j, b), (2j+1, -c) and row 2i+1 holds
// (2j, c), (2j+1, b) for each entry b + ic of row i at column j, in the
// order of row i; so [re; im] rows give Re and Im of (A x)_i, and the
// transposed form gives A^H x on the same pairs.
extern "C" int propack_zcsr_expand(int m, int n, const int64_t *rowptr, const int32_t *colidx,
                                   const propack_z16 *val, int64_t *rowptr2, int32_t *colidx2, double *val2)
{
    if (m < 0 || n < 0 || !rowptr || !rowptr2 || m > INT32_MAX / 2 || n > INT32_MAX / 2) return PROPACK_ERR_ARG;
    const int64_t nnz = rowptr[m];
    if (nnz < 0 || 4 * nnz >= (int64_t)INT32_MAX) return PROPACK_ERR_ARG;
    if (nnz > 0 && (!colidx || !val || !colidx2 || !val2)) return PROPACK_ERR_ARG;
    if (rowptr[0] != 0) return PROPACK_ERR_ARG;
    for (int i = 0; i < m; i++)
        if (rowptr[i + 1] < rowptr[i]) return PROPACK_ERR_ARG;
    rowptr2[0] = 0;
    for (int i = 0; i < m; i++) {
        const int64_t p0 = rowptr[i], p1 = rowptr[i + 1], len = p1 - p0;
        const int64_t r0 = 4 * p0, r1 = r0 + 2 * len;  // starts of rows 2i and 2i+1
        rowptr2[2 * i + 1] = r1;
        rowptr2[2 * i + 2] = r1 + 2 * len;
        for (int64_t e = p0; e < p1; e++) {
            if (colidx[e] < 0 || colidx[e] >= n) return PROPACK_ERR_ARG;
            const int64_t q = 2 * (e - p0);
            const int32_t j2 = 2 * colidx[e];
            const double b = val[e].re, c = val[e].im;
            colidx2[r0 + q] = j2;
            val2[r0 + q] = b;
            colidx2[r0 + q + 1] = j2 + 1;
            val2[r0 + q + 1] = -c;
            colidx2[r1 + q] = j2;
            val2[r1 + q] = c;
            colidx2[r1 + q + 1] = j2 + 1;
            val2[r1 + q + 1] = b;
        }
    }
    return 0;
}

// propack_set_zcsr_form: 0 native complex CSR (default), 1 the real
// 2x2-block form; applies to operators created afterwards
static std::atomic<int> g_zform{0};
extern "C" int propack_set_zcsr_form(int form)
{
    if (form != 0 && form != 1) return PROPACK_ERR_ARG;
    g_zform.store(form);
    return 0;
}

extern "C" int propack_zcsr_create(int m, int n, const int64_t *rowptr, const int32_t *colidx,
                                   const propack_z16 *val, int64_t *handle)
{
    if (m <= 0 || n <= 0 || !rowptr || !handle) {
        set_error("invalid argument to propack_zcsr_create");
        return PROPACK_ERR_ARG;
    }
    if (g_zform.load() == 0) {
        try {
            return create_zoperator(m, n, rowptr, colidx, val, handle);
        } catch (const CudaFailure &) {
            return PROPACK_ERR_CUDA;
        } catch (const ArgFailure &) {
            if (g_err.empty()) set_error("invalid argument to propack_zcsr_create");
            return PROPACK_ERR_ARG;
        }
    }
    const int64_t nnz = rowptr[m];
    if (nnz < 0 || 4 * nnz >= (int64_t)INT32_MAX) {
        set_error("complex operator has 2^29 or more nonzeros (its real form 2^31)");
        return PROPACK_ERR_ARG;
    }
    // the expansion checks row pointers and column indices on the host; the
    // real form is checked again on the device by propack_csr_create
    std::vector<int64_t> p2(2 * (size_t)m + 1);
    std::vector<int32_t> i2(std::max<int64_t>(4 * nnz, 1));
    std::vector<double> v2(std::max<int64_t>(4 * nnz, 1));
    if (propack_zcsr_expand(m, n, rowptr, colidx, val, p2.data(), i2.data(), v2.data()) != 0) {
        set_error(rowptr[0] != 0 ? "row pointers are not monotone from 0 to nnz"
                                 : "row pointers are not monotone from 0 to nnz, or a column index is out of range");
        return PROPACK_ERR_ARG;
    }
    const int rc = propack_csr_create(2 * m, 2 * n, p2.data(), i2.data(), v2.data(), 0, nullptr, nullptr, nullptr,
                                      nullptr, nullptr, nullptr, nullptr, handle);
    if (rc != 0) return rc;
    Operator *op = lookup_operator(*handle);
    if (op) op->cplx = 1;
    return 0;
}

// ------------------------------------------------------ gather ceiling
// The rate at which this GPU serves random 8-byte reads from a vector that
// stays in L2, with their 12-byte (index, value) stream: the ceiling of a
// sparse product whose columns are uniformly random, which no row schedule
// can beat.  Flat, no rows: every thread takes GP_U independent entries at
// a time (grid stride), loads their indices and values, then their x
// values, and accumulates; the index stream is a hash of the position, so
// every read stays inside x.
constexpr int GP_U = 4;
__global__ void k_gp_fill(int *idx, double *val, int64_t nnz, int n)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
        unsigned long long z = (unsigned long long)e * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
        z ^= z >> 31;
        z *= 0xBF58476D1CE4E5B9ull;
        z ^= z >> 29;
        idx[e] = (int)(z % (unsigned long long)n);
        val[e] = 1.0 + (double)(e & 7);
    }
}
__global__ void k_gp_fill_x(double *x, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = 1.0 / (1.0 + i);
}
__global__ void __launch_bounds__(BS) k_gp_gather(const int *__restrict__ idx, const double *__restrict__ val,
                                                  const double *__restrict__ x, int64_t nnz, double *out)
{
    double s = 0.0;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, st = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = t; i < nnz; i += st * GP_U) {
        int c[GP_U];
        double v[GP_U];
#pragma unroll
        for (int u = 0; u < GP_U; u++) {
            const int64_t k = i + u * st;
            c[u] = k < nnz ? idx[k] : 0;
            v[u] = k < nnz ? val[k] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < GP_U; u++) s = fma(v[u], x[c[u]], s);
    }
    if (s == -1.0) *out = s;  // keeps the loads; never true for the positive data
}

extern "C" int propack_gather_ceiling(int n, int64_t nnz, float *ms)
{
    if (n <= 0 || nnz <= 0 || !ms) return PROPACK_ERR_ARG;
    int *idx = nullptr;
    double *val = nullptr, *x = nullptr, *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t s = nullptr;
    try {
        PGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        idx = (int *)pool_alloc(sizeof(int) * nnz, s);
        val = (double *)pool_alloc(sizeof(double) * nnz, s);
        x = (double *)pool_alloc(sizeof(double) * n, s);
        out = (double *)pool_alloc(sizeof(double), s);
        const int g = device_info().nb;
        k_gp_fill<<<g, BS, 0, s>>>(idx, val, nnz, n);
        k_gp_fill_x<<<g, BS, 0, s>>>(x, n);
        PGB_CUDA(cudaEventCreate(&e0));
        PGB_CUDA(cudaEventCreate(&e1));
        std::vector<float> t;
        for (int r = 0; r < 8; r++) {
            PGB_CUDA(cudaEventRecord(e0, s));
            k_gp_gather<<<g, BS, 0, s>>>(idx, val, x, nnz, out);
            PGB_CUDA(cudaEventRecord(e1, s));
            PGB_CUDA(cudaEventSynchronize(e1));
            float v = 0.f;
            PGB_CUDA(cudaEventElapsedTime(&v, e0, e1));
            if (r >= 3) t.push_back(v);
        }
        std::sort(t.begin(), t.end());
        *ms = t[t.size() / 2];
        pool_free(idx, s);
        pool_free(val, s);
        pool_free(x, s);
        pool_free(out, s);
        PGB_CUDA(cudaStreamSynchronize(s));
    } catch (const CudaFailure &) {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (s) cudaStreamDestroy(s);
        return PROPACK_ERR_CUDA;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    return 0;
}

extern "C" int propack_release_memory(void)
{
    try {
        PGB_CUDA(cudaDeviceSynchronize());
        PGB_CUDA(cudaMemPoolTrimTo(lib_pool(), 0));
        release_bounce_buffers();
    } catch (const CudaFailure &) {
        return PROPACK_ERR_CUDA;
    }
    return 0;
}

extern "C" int propack_set_spmv_schedule(int mode)
{
    if (mode < 0 || mode > 3) return PROPACK_ERR_ARG;
    g_sched.store(mode);
    return 0;
}

extern "C" int propack_csr_schedule(int64_t handle, int *sched, float *tuned_ms)
{
    Operator *op = lookup_operator(handle);
    if (!op) return PROPACK_ERR_HANDLE;
    const Csr *M[2] = {&op->fwd, &op->adj};
    for (int i = 0; i < 2; i++) {
        if (sched) sched[i] = M[i]->short_rows;
        if (tuned_ms) {
            tuned_ms[2 * i] = M[i]->tuned_ms[0];
            tuned_ms[2 * i + 1] = M[i]->tuned_ms[1];
        }
    }
    return 0;
}

extern "C" void propack_handle_to_iparm(int64_t handle, int *iparm)
{
    iparm[0] = (int)(uint32_t)((uint64_t)handle & 0xffffffffu);
    iparm[1] = (int)(uint32_t)((uint64_t)handle >> 32);
}

extern "C" void propack_gpu_csr_saprod_(const char *transa, const int *m, const int *n, const float *x, float *y,
                                        float *dparm, int *iparm, size_t transa_len)
{
    (void)dparm;
    const bool t = (transa[0] == 't' || transa[0] == 'T');
    const int nin = t ? *m : *n, nout = t ? *n : *m;
    std::vector<double> xd(std::max(nin, 1)), yd(std::max(nout, 1));
    for (int i = 0; i < nin; i++) xd[i] = x[i];
    propack_gpu_csr_aprod_(transa, m, n, xd.data(), yd.data(), nullptr, iparm, transa_len);
    for (int i = 0; i < nout; i++) y[i] = (float)yd[i];
}

extern "C" void propack_gpu_csr_zaprod_(const char *transa, const int *m, const int *n, const propack_z16 *x,
                                        propack_z16 *y, propack_z16 *zparm, int *iparm, size_t transa_len)
{
    (void)zparm;
    Operator *op = lookup_operator(handle_from_iparm(iparm));
    if (!op || !op->cplx) { set_error("propack_gpu_csr_zaprod_: iparm holds no live complex operator"); return; }
    if (op->cplx == 2) {
        if (op->m != *m || op->n != *n) {
            set_error("propack_gpu_csr_zaprod_: m, n do not match the operator");
            return;
        }
        const bool t = !(transa[0] == 'n' || transa[0] == 'N');
        const int nin = t ? *m : *n, nout = t ? *n : *m;
        try {
            cudaStream_t s;
            PGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            double2 *dx = nullptr, *dy = nullptr;
            dx = static_cast<decltype(dx)>(pool_alloc(sizeof(double2) * nin, s));
            dy = static_cast<decltype(dy)>(pool_alloc(sizeof(double2) * nout, s));
            PGB_CUDA(cudaMemcpyAsync(dx, x, sizeof(double2) * nin, cudaMemcpyHostToDevice, s));
            op_zapply(*op, t, dx, dy, s);
            PGB_CUDA(cudaMemcpyAsync(y, dy, sizeof(double2) * nout, cudaMemcpyDeviceToHost, s));
            pool_free(dx, s);
            pool_free(dy, s);
            PGB_CUDA(cudaStreamSynchronize(s));
            PGB_CUDA(cudaStreamDestroy(s));
        } catch (...) {
        }
        return;
    }
    // the real form is 2m x 2n: 'n' gives A x, anything else A^H x
    const int m2 = 2 * *m, n2 = 2 * *n;
    const char t = (transa[0] == 'n' || transa[0] == 'N') ? 'n' : 't';
    propack_gpu_csr_aprod_(&t, &m2, &n2, (const double *)x, (double *)y, nullptr, iparm, transa_len);
}

extern "C" void propack_gpu_csr_aprod_(const char *transa, const int *m, const int *n, const double *x, double *y,
                                       double *dparm, int *iparm, size_t transa_len)
{
    (void)dparm; (void)transa_len;
    Operator *op = lookup_operator(handle_from_iparm(iparm));
    if (!op) { set_error("propack_gpu_csr_aprod_: iparm holds no live operator"); return; }
    if (op->cplx == 2) { set_error("propack_gpu_csr_aprod_: a complex operator needs propack_gpu_csr_zaprod_"); return; }
    if (op->m != *m || op->n != *n) { set_error("propack_gpu_csr_aprod_: m, n do not match the operator"); return; }
    const bool t = (transa[0] == 't' || transa[0] == 'T');
    const int nin = t ? *m : *n, nout = t ? *n : *m;
    try {
        cudaStream_t s;
        PGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        double *dx = nullptr, *dy = nullptr;
        dx = static_cast<decltype(dx)>(pool_alloc(sizeof(double) * nin, s));
        dy = static_cast<decltype(dy)>(pool_alloc(sizeof(double) * nout, s));
        PGB_CUDA(cudaMemcpyAsync(dx, x, sizeof(double) * nin, cudaMemcpyHostToDevice, s));
        op_apply<double>(*op, t, dx, dy, s);
        PGB_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * nout, cudaMemcpyDeviceToHost, s));
        pool_free(dx, s);
        pool_free(dy, s);
        PGB_CUDA(cudaStreamSynchronize(s));
        PGB_CUDA(cudaStreamDestroy(s));
    } catch (...) {
    }
}

extern "C" const char *propack_last_error(void) { return pgb::last_error(); }

namespace pgb {
void prof_reset();
void prof_get(double *ms, int64_t *cnt, int n);
}
extern "C" void propack_set_profiling(int on)
{
    pgb::g_prof_on = on ? 1 : 0;
    pgb::prof_reset();
}
extern "C" int propack_get_profile(double *total_ms, int64_t *launches, int n)
{
    pgb::prof_collect();
    pgb::prof_get(total_ms, launches, n);
    return pgb::PK_N;
}
