// pgb_noalloc.cu -- applying the device operator without allocating device
// memory.
//
// Who needs this: callers that may not call cudaMalloc / cudaFree (or any
// routine that allocates) while they run.  Typical cases are code on a
// latency-critical path where an allocation's implicit device
// synchronisation or allocator lock is unacceptable, code that runs while
// another component owns all free device memory under a fixed cap, and
// code that has to stay replayable with the same addresses every time.
// The regular entry point propack_gpu_csr_aprod_ allocates its device
// vectors per call; this one takes device pointers from the caller and
// keeps its only scratch -- the partial sums of the low-rank prepass and
// the resulting coefficients z -- in one fixed array in device memory that
// every GPU which loads the library holds until the process exits.
#include <mutex>

#include "../../include/propack_gb300.h"
#include "pgb.cuh"

namespace pgb {

void op_spmv_plain_launch(const Csr &A, const double *x, const double *z, double *y, cudaStream_t s);

// The shared scratch: PROPACK_NOALLOC_MAX_DOUBLES doubles (512 KiB).  Layout
// for an operator of rank r whose thin transpose needs `segs` segments per
// row: [0, r) the coefficients z, [r, r + r*segs) the segment partials, and
// the last element reinterpreted as the last-CTA ticket.
static __device__ __align__(256) double g_noalloc_scratch[PROPACK_NOALLOC_MAX_DOUBLES];

// z[c] = w[c] * sum(thin row c . x), segments of NNZ_PB per CTA, partials in
// the static scratch (the same reduction as the allocating prepass).
__global__ void __launch_bounds__(BS) k_thin_noalloc(Csr T, const double *__restrict__ x, const double *w, int r)
{
    __shared__ double sred[32];
    double *z = g_noalloc_scratch;
    double *zpart = g_noalloc_scratch + r;
    unsigned int *ticket = reinterpret_cast<unsigned int *>(g_noalloc_scratch + (PROPACK_NOALLOC_MAX_DOUBLES - 1));
    const int nseg = T.segs;
    for (int t = blockIdx.x; t < T.rows * nseg; t += gridDim.x) {
        const int c = t / nseg, sg = t % nseg;
        const int a = T.ptr[c] + sg * NNZ_PB;
        const int b = min(T.ptr[c + 1], a + NNZ_PB);
        double acc = 0.0;
        for (int e = a + threadIdx.x; e < b; e += BS) acc += T.val[e] * x[T.idx[e]];
        acc = block_sum<BS>(acc, sred);
        if (threadIdx.x == 0) zpart[t] = acc;
    }
    if (last_cta(ticket)) {
        for (int c = threadIdx.x; c < T.rows; c += BS) {
            double s = 0.0;
            for (int sg = 0; sg < nseg; sg++) s += zpart[c * nseg + sg];
            z[c] = w[c] * s;
        }
    }
}

// Device address of the scratch array for each device, looked up once
// with that device current (cudaGetSymbolAddress allocates nothing).
static double *g_scratch_addr[64];
static bool g_scratch_ready[64];
static std::mutex g_scratch_mu;

static double *scratch_address(int dev)
{
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (dev < 0 || dev >= 64) {
        set_error("propack_csr_apply_noalloc: device index out of range");
        throw ArgFailure();
    }
    if (!g_scratch_ready[dev]) {
        double *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error(std::string("propack_csr_apply_noalloc: cudaGetSymbolAddress failed: ") +
                      cudaGetErrorString(e));
            throw CudaFailure();
        }
        g_scratch_addr[dev] = p;
        g_scratch_ready[dev] = true;
    }
    return g_scratch_addr[dev];
}

// a pointer the kernels may dereference on device `dev`: device memory of
// that device, managed memory, or host memory mapped for it (its
// devicePointer is the pointer itself).  cudaPointerGetAttributes
// allocates nothing; a plain host pointer is refused here instead of
// faulting in a kernel.
static bool usable_on(const void *p, int dev)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (at.type == cudaMemoryTypeManaged) return true;
    if (at.type == cudaMemoryTypeDevice) return at.device == dev;
    if (at.type == cudaMemoryTypeHost) return at.devicePointer == p;
    return false;
}

static int apply_noalloc(int64_t handle, int trans, const double *x, double *y, cudaStream_t s)
{
    const Operator *op = lookup_operator(handle);
    if (!op) {
        set_error("propack_csr_apply_noalloc: no live operator with this handle");
        return PROPACK_ERR_HANDLE;
    }
    if (!x || !y) {
        set_error("propack_csr_apply_noalloc: x and y must be device pointers");
        return PROPACK_ERR_ARG;
    }
    int dev = 0;
    PGB_CUDA(cudaGetDevice(&dev));
    if (dev != op->device) {
        set_error("propack_csr_apply_noalloc: the operator lives on another device than the current one");
        return PROPACK_ERR_ARG;
    }
    if (!usable_on(x, dev) || !usable_on(y, dev)) {
        set_error("propack_csr_apply_noalloc: x and y must be device (or managed) memory of the operator's device");
        return PROPACK_ERR_ARG;
    }
    if (op->cplx == 2) {
        // a native complex operator: x and y hold (re, im) pairs, read as
        // 16-byte vectors
        if ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y)) & 15u) {
            set_error("propack_csr_apply_noalloc: complex x and y must be 16-byte aligned");
            return PROPACK_ERR_ARG;
        }
        op_zspmv_plain_launch(trans ? op->adj : op->fwd, reinterpret_cast<const double2 *>(x),
                              reinterpret_cast<double2 *>(y), s);
        PGB_CUDA(cudaGetLastError());
        return 0;
    }
    double *base = scratch_address(dev);
    const Csr &A = trans ? op->adj : op->fwd;
    const double *z = nullptr;
    if (op->r > 0) {
        const Csr &T = trans ? op->thin_l : op->thin_r;
        const long long need = (long long)op->r * (1 + T.segs) + 1;
        if (need > PROPACK_NOALLOC_MAX_DOUBLES) {
            set_error("propack_csr_apply_noalloc: the operator's low-rank term needs " + std::to_string(need) +
                      " doubles of scratch, more than the fixed " + std::to_string(PROPACK_NOALLOC_MAX_DOUBLES));
            return PROPACK_ERR_ARG;
        }
        // the ticket must start at zero on every call
        PGB_CUDA(cudaMemsetAsync(base + (PROPACK_NOALLOC_MAX_DOUBLES - 1), 0, sizeof(double), s));
        const int nt = std::max(1, T.rows * T.segs);
        k_thin_noalloc<<<std::min(nt, device_info().nb), BS, 0, s>>>(T, x, op->w, op->r);
        PGB_LAUNCHED();
        PGB_CUDA(cudaGetLastError());
        z = base;
    }
    op_spmv_plain_launch(A, x, z, y, s);
    PGB_CUDA(cudaGetLastError());
    return 0;
}

}  // namespace pgb

extern "C" int propack_csr_apply_noalloc(int64_t handle, int trans, const double *x, double *y, void *stream)
{
    try {
        return pgb::apply_noalloc(handle, trans, x, y, (cudaStream_t)stream);
    } catch (const pgb::CudaFailure &) {
        return PROPACK_ERR_CUDA;
    } catch (const pgb::ArgFailure &) {
        return PROPACK_ERR_ARG;
    }
}
