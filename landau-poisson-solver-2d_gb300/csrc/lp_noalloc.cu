// Allocation-free moment-conserving projection (lp_conserve_noalloc).
//
// Some callers cannot allocate device memory at the moment they need the
// projection: code that hands all device memory to another framework's pool
// and may not call cudaMalloc behind its back, or a time-critical loop where
// cudaMalloc/cudaFree (which can synchronise the whole device) are not
// allowed.  For them this file keeps the projection's scratch -- the per-chunk
// partial dot products and the five Lagrange multipliers of every cell -- in
// one fixed device array compiled into the library, so a call needs no
// allocation at all: the caller passes the mode arrays, the constraint rows
// and the inverse Gram matrix in device memory it already owns.
//
// The array holds LP_NOALLOC_MAX_CELLS cells' worth of scratch (about
// 2.8 MB); every GPU that loads this library keeps it until the process
// exits.  Calls share it: two calls whose kernels overlap on the GPU (on
// different streams, or from different host threads) race on it and give
// wrong results; serialise them.  Each call overwrites every scratch entry it
// reads, so nothing carries over from the previous call.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "lp_gb300.h"

namespace {

constexpr int kChunks = 16;       // partial sums per cell
constexpr int kMaxDevices = 64;
constexpr size_t kScratchDoubles = (size_t)LP_NOALLOC_MAX_CELLS * (kChunks * 5 + 5);

// The scratch: partial sums [cell][chunk][5], then multipliers [cell][5].
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// Device address of g_noalloc_scratch per device ordinal, looked up once per
// device with that device current.  A cudaDeviceReset unloads the module and
// leaves this address stale, so the entry point must not be used across one.
double *g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

// A kernel launched as a programmatic dependent (inside a caller's graph
// whose edges allow early launch) reads nothing before its predecessors have
// completed; under an ordinary launch this returns at once.
__device__ __forceinline__ void na_grid_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// t_m = sum over the chunk of Re/Im(q) times the constraint rows
// (conserveAllMoments, source/conservationRoutines.cpp:109-117), one block per
// (chunk, cell), reference layout q[cell][n3].
__global__ void k_na_partial(const double2 *__restrict__ q, const double *__restrict__ c1,
                             const double *__restrict__ c2, int n3, double *__restrict__ part) {
    na_grid_wait();
    __shared__ double red[5][256];
    const int cell = blockIdx.y, k = blockIdx.x, t = threadIdx.x;
    const int cs = (n3 + kChunks - 1) / kChunks, p0 = k * cs, p1 = min(n3, p0 + cs);
    const double2 *qc = q + (long long)cell * n3;
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0;
    for (int pt = p0 + t; pt < p1; pt += 256) {
        const double2 v = qc[pt];
        s0 += v.x * c1[pt];
        s1 += v.y * c2[n3 + pt];
        s2 += v.y * c2[2 * n3 + pt];
        s3 += v.y * c2[3 * n3 + pt];
        s4 += v.x * c1[4 * n3 + pt];
    }
    red[0][t] = s0; red[1][t] = s1; red[2][t] = s2; red[3][t] = s3; red[4][t] = s4;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w)
            for (int m = 0; m < 5; ++m) red[m][t] += red[m][t + w];
        __syncthreads();
    }
    if (t < 5) part[((long long)cell * kChunks + k) * 5 + t] = red[t][0];
}

// lambda = (C C^T)^-1 t per cell (solveWithCCt, conservationRoutines.cpp:49-55).
__global__ void k_na_lambda(const double *__restrict__ part, const double *__restrict__ cct, int ncell,
                            double *__restrict__ lam) {
    na_grid_wait();
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncell) return;
    double t[5] = {0, 0, 0, 0, 0};
    for (int k = 0; k < kChunks; ++k)
        for (int m = 0; m < 5; ++m) t[m] += part[((long long)cell * kChunks + k) * 5 + m];
    for (int i = 0; i < 5; ++i) {
        double s = 0.;
        for (int j = 0; j < 5; ++j) s += cct[j + i * 5] * t[j];
        lam[5 * cell + i] = s;
    }
}

// q -= C^T lambda (conservationRoutines.cpp:121-126).
__global__ void k_na_apply(double2 *__restrict__ q, const double *__restrict__ c1, const double *__restrict__ c2,
                           const double *__restrict__ lam, int n3, long long total) {
    na_grid_wait();
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= total) return;
    const int cell = (int)(tid / n3), pt = (int)(tid % n3);
    const double *l = lam + 5 * cell;
    double2 v = q[tid];
    v.x -= (c1[pt] * l[0] + c1[4 * n3 + pt] * l[4]);
    v.y -= (c2[n3 + pt] * l[1] + c2[2 * n3 + pt] * l[2] + c2[3 * n3 + pt] * l[3]);
    q[tid] = v;
}

}  // namespace

extern "C" lp_status lp_conserve_noalloc(double *qhat_dev, int ncell, int n3, const double *c1_dev,
                                         const double *c2_dev, const double *cct_inv_dev, void *cuda_stream) {
    if (!qhat_dev || !c1_dev || !c2_dev || !cct_inv_dev) return LP_ERR_INVALID;
    if (ncell < 1 || ncell > LP_NOALLOC_MAX_CELLS || n3 < 1 || n3 > 32 * 32 * 32) return LP_ERR_INVALID;
    // the mode array is read as double2 (16-byte) values, the rows as doubles
    if (reinterpret_cast<uintptr_t>(qhat_dev) % 16 || reinterpret_cast<uintptr_t>(c1_dev) % 8 ||
        reinterpret_cast<uintptr_t>(c2_dev) % 8 || reinterpret_cast<uintptr_t>(cct_inv_dev) % 8)
        return LP_ERR_INVALID;
    // an error left pending by the caller's earlier CUDA work is reported, not
    // cleared, and nothing is launched
    if (cudaPeekAtLastError() != cudaSuccess) return LP_ERR_CUDA;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return LP_ERR_NO_DEVICE;
    }
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                return LP_ERR_CUDA;
            }
            g_scratch_addr[dev] = static_cast<double *>(p);
        }
        scratch = g_scratch_addr[dev];
    }
    double *part = scratch;
    double *lam = scratch + (size_t)LP_NOALLOC_MAX_CELLS * kChunks * 5;
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    double2 *q = reinterpret_cast<double2 *>(qhat_dev);
    // each launch is checked before the next; a failed launch's own error is
    // the only one cleared here
    k_na_partial<<<dim3(kChunks, ncell), 256, 0, st>>>(q, c1_dev, c2_dev, n3, part);
    if (cudaGetLastError() != cudaSuccess) return LP_ERR_CUDA;
    k_na_lambda<<<(ncell + 127) / 128, 128, 0, st>>>(part, cct_inv_dev, ncell, lam);
    if (cudaGetLastError() != cudaSuccess) return LP_ERR_CUDA;
    const long long total = (long long)ncell * n3;
    k_na_apply<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(q, c1_dev, c2_dev, lam, n3, total);
    return cudaGetLastError() == cudaSuccess ? LP_OK : LP_ERR_CUDA;
}
