// The axis-3 pass of the mixed path's DG projection (IntModes, source/
// collisionRoutines_1.cpp:364-505, applied in RK4 at C:867-905) on the
// tensor cores.
//
// Per (pencil (k1, k2), cell) the pass forms the RK4 combination
// x(k3) = nu (q0/2 + (q1 + q2 + q3)/6) of the four stage mode arrays (with
// the stages' deferred conservation corrections q_s -= C^T lambda_s) and
// contracts it with the three per-axis factor tables T0, T1, T2 ([n][nv]
// complex each): Y_a(j3) = sum_k3 T_a(k3, j3) x(k3).  Over 128 (pencil, cell)
// rows at a time that is one real GEMM with a shared operand:
//
//   A (128 x 2n):  [Re x(0..n-1) | Im x(0..n-1)] per row,
//   B (2n x 6 nv): columns (a, j, re/im) = [Tr; -Ti] and [Ti; Tr],
//   D = A B (128 x 6 nv, FP32 in tensor memory).
//
// FP32 operands go through three TF32 products (hi hi + hi lo + lo hi, the
// operands split into a TF32 head and a TF32 tail), accumulated in FP32:
// about 2^-21 relative per product, against 2^-24 for the CUDA-core pass
// this replaces.  B (both splits, in the shared-memory layout of the MMA)
// is built once on the host and brought in by one bulk copy; A is formed,
// split and stored by the block's 128 threads, one row each; one thread
// issues the 3 x (2n / 8) MMAs; the 128 threads read back their row of D
// and store Y cell-minor (each warp 32 consecutive cells, 256-byte stores).
#include "lp_kernels.cuh"
#include "lp_dev.cuh"
#include "lp_tc.cuh"

#include <cstring>
#include <type_traits>

namespace lp {
namespace {

constexpr int kRows = 128;

// row r of tile `tile` -> (pencil, cell): the rows run over (pencil, cell)
// pairs in the arrays' own order, 128 per tile; Bp is a multiple of 32, so
// the 32 rows of a warp are 32 consecutive cells of one pencil
__device__ __forceinline__ void tile_row(int tile, int r, int Bp, int &pid, int &c) {
    const long long g = (long long)tile * kRows + r;
    pid = (int)(g / Bp);
    c = (int)(g % Bp);
}

template <int N, typename QT>
__global__ void __launch_bounds__(kRows) k_pj3_tc(const QT *__restrict__ q0, const QT *__restrict__ q1,
                                                  const QT *__restrict__ q2, const QT *__restrict__ q3, double nu,
                                                  const double *__restrict__ cnu, const float *__restrict__ btab,
                                                  int nv, int NP, int tcols, int Bp, float2 *__restrict__ Y,
                                                  const float *__restrict__ cf, const double *__restrict__ lam4,
                                                  int *__restrict__ err) {
    constexpr int K = 2 * N, KC = K / 4;  // K of the real GEMM, its 16-byte core columns
    extern __shared__ __align__(1024) unsigned char sm[];
    const uint32_t bbytes = (uint32_t)NP * K * 4;
    unsigned char *Bhi = sm, *Blo = sm + bbytes, *Ahi = sm + 2 * bbytes, *Alo = Ahi + kRows * K * 4;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, w = t >> 5;
    if (t == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (w == 0) tc::tmem_alloc(&tslot, (uint32_t)tcols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;
    if (t == 0) {
        tc::mbar_expect_tx(&mbar[0], 2 * bbytes);
        tc::bulk_g2s(Bhi, btab, 2 * bbytes, &mbar[0]);
    }
    // this thread's row: the RK4 combination of its pencil along k3
    int pid, c;
    tile_row(blockIdx.x, t, Bp, pid, c);
    const double nuc = cnu ? cnu[c] : nu;
    float xr[N], xi[N];
    const long long b = (long long)pid * N * Bp + c;
    if (cf) {
        constexpr int n3 = N * N * N;
        float l[4][5];
#pragma unroll
        for (int s = 0; s < 4; ++s)
#pragma unroll
            for (int j = 0; j < 5; ++j) l[s][j] = (float)lam4[(s * 5 + j) * Bp + c];
        const float nuf = (float)nuc;
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const long long o = b + (long long)k * Bp;
            const int pt = pid * N + k;
            const float r0 = cf[pt], r1 = cf[n3 + pt], r2 = cf[2 * n3 + pt], r3 = cf[3 * n3 + pt], r4 = cf[4 * n3 + pt];
            const QT qs[4] = {q0[o], q1[o], q2[o], q3[o]};
            float vr[4], vi[4];
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                vr[s] = (float)qs[s].x - (r0 * l[s][0] + r4 * l[s][4]);
                vi[s] = (float)qs[s].y - (r1 * l[s][1] + r2 * l[s][2] + r3 * l[s][3]);
            }
            xr[k] = nuf * (0.5f * vr[0] + (vr[1] + vr[2] + vr[3]) * (1.f / 6.f));
            xi[k] = nuf * (0.5f * vi[0] + (vi[1] + vi[2] + vi[3]) * (1.f / 6.f));
        }
    } else {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const long long o = b + (long long)k * Bp;
            const QT a = q0[o], e = q1[o], d = q2[o], g = q3[o];
            xr[k] = (float)(nuc * (0.5 * a.x + (e.x + d.x + g.x) * (1. / 6.)));
            xi[k] = (float)(nuc * (0.5 * a.y + (e.y + d.y + g.y) * (1. / 6.)));
        }
    }
    // TF32 head and tail of the row, 16 bytes (4 elements of K) per store
#pragma unroll
    for (int k = 0; k < N; k += 4) {
        float4 hr, lr, hi4, li4;
        float *phr = &hr.x, *plr = &lr.x, *phi = &hi4.x, *pli = &li4.x;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float a = xr[k + u], bq = xi[k + u];
            phr[u] = tc::tf32_rna(a);
            plr[u] = tc::tf32_rna(a - phr[u]);
            phi[u] = tc::tf32_rna(bq);
            pli[u] = tc::tf32_rna(bq - phi[u]);
        }
        *reinterpret_cast<float4 *>(Ahi + tc::core_off(t, k, KC)) = hr;
        *reinterpret_cast<float4 *>(Alo + tc::core_off(t, k, KC)) = lr;
        *reinterpret_cast<float4 *>(Ahi + tc::core_off(t, N + k, KC)) = hi4;
        *reinterpret_cast<float4 *>(Alo + tc::core_off(t, N + k, KC)) = li4;
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (t == 0) {
        const bool have_b = tc::mbar_wait(&mbar[0], 0);
        if (have_b) {
            const uint32_t idesc = tc::idesc_tf32(kRows, NP);
            const uint32_t lbo = 128, sbo = KC * 128;
            const unsigned char *As[3] = {Ahi, Ahi, Alo}, *Bs[3] = {Bhi, Blo, Bhi};
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int ks = 0; ks < K / 8; ++ks)
                    tc::mma_tf32(tmem, tc::sdesc(tc::smem_u32(As[p]) + ks * 256, lbo, sbo),
                                 tc::sdesc(tc::smem_u32(Bs[p]) + ks * 256, lbo, sbo), idesc, p > 0 || ks > 0);
        } else {
            atomicExch(err, 1);
            tc::mbar_wait(&mbar[0], 0);  // give the bulk copy another bounded wait before leaving
        }
        tc::mma_commit(&mbar[1]);
    }
    const bool done = tc::mbar_wait(&mbar[1], 0);
    if (!done) atomicExch(err, 2);
    tc::fence_after_sync();
    if (done) {
        const int ncol = 6 * nv;
        const uint32_t lane_base = tmem + ((uint32_t)(32 * w) << 16);
        for (int c0 = 0; c0 < ncol; c0 += 16) {
            float v[16];
            tc::tmem_ld16(lane_base + (uint32_t)c0, v);
#pragma unroll
            for (int u = 0; u < 16; u += 2) {
                const int col = c0 + u;
                if (col < ncol) {
                    const int aj = col >> 1, a = aj / nv, j = aj - a * nv;
                    Y[(((long long)a * N * N + pid) * nv + j) * Bp + c] = make_float2(v[u], v[u + 1]);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (w == 0) tc::tmem_free(tmem, (uint32_t)tcols);
}

}  // namespace

int pj3_tc_np(int nv) { return ((6 * nv + 15) / 16) * 16; }

bool pj3_tc_supported(int n, int nv, int Bp) {
    if (!(n == 8 || n == 16 || n == 24 || n == 32)) return false;
    if (pj3_tc_np(nv) > 256) return false;
    if (Bp < 32 || Bp % 32) return false;
    return ((long long)n * n * Bp) % kRows == 0;
}

size_t pj3_tc_table_floats(int n, int nv) { return (size_t)2 * pj3_tc_np(nv) * 2 * n; }

// B = [Tr; -Ti | Ti; Tr] per (table a, output j), split into TF32 head and
// tail, in the K-major core-matrix layout of the MMA (head, then tail).
static float tf32_round_host(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x1000u) & ~0x1FFFu;  // round to nearest at mantissa bit 13, ties away from zero
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

void pj3_tc_table(const float *tfac, int n, int nv, std::vector<float> &out) {
    const int K = 2 * n, KC = K / 4, NP = pj3_tc_np(nv);
    out.assign(pj3_tc_table_floats(n, nv), 0.f);
    float *hi = out.data(), *lo = out.data() + (size_t)NP * K;
    for (int a = 0; a < 3; ++a)
        for (int j = 0; j < nv; ++j)
            for (int k = 0; k < n; ++k) {
                const size_t t = ((size_t)a * n + k) * nv + j;
                const float tr = tfac[2 * t], ti = tfac[2 * t + 1];
                const int cre = 2 * (a * nv + j), cim = cre + 1;
                const float vals[4] = {tr, -ti, ti, tr};  // (cre, k), (cre, n+k), (cim, k), (cim, n+k)
                const int rows[4] = {cre, cre, cim, cim}, ks[4] = {k, n + k, k, n + k};
                for (int e = 0; e < 4; ++e) {
                    const float h = tf32_round_host(vals[e]);
                    const float l = tf32_round_host(vals[e] - h);
                    const int off = tc::core_off(rows[e], ks[e], KC) / 4;
                    hi[off] = h;
                    lo[off] = l;
                }
            }
}

size_t pj3_tc_smem(int n, int nv) { return (size_t)2 * pj3_tc_np(nv) * 2 * n * 4 + (size_t)2 * kRows * 2 * n * 4; }

template <int N, typename QT>
static cudaError_t pj3_tc_go(const QT *q0, const QT *q1, const QT *q2, const QT *q3, double nu, const double *cnu,
                             const float *btab, int nv, int Bp, float2 *Y, const float *cf, const double *lam4,
                             int *err, cudaStream_t st) {
    const int NP = pj3_tc_np(nv);
    const int tcols = NP <= 32 ? 32 : (NP <= 64 ? 64 : (NP <= 128 ? 128 : 256));
    const size_t smem = pj3_tc_smem(N, nv);
    cudaError_t e = cudaFuncSetAttribute(k_pj3_tc<N, QT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int tiles = (int)((long long)N * N * Bp / kRows);
    k_pj3_tc<N, QT><<<tiles, kRows, smem, st>>>(q0, q1, q2, q3, nu, cnu, btab, nv, NP, tcols, Bp, Y, cf, lam4, err);
    return cudaGetLastError();
}

template <typename QT>
cudaError_t launch_pj3_tc(const QT *q0, const QT *q1, const QT *q2, const QT *q3, double nu, const double *cnu,
                          const float *btab, int n, int nv, int Bp, float2 *Y, const float *cf, const double *lam4,
                          int *err, cudaStream_t st) {
    if (!pj3_tc_supported(n, nv, Bp) || !btab || !err) return cudaErrorInvalidValue;
    if (reinterpret_cast<uintptr_t>(btab) % 16) return cudaErrorInvalidValue;
    switch (n) {
    case 8: return pj3_tc_go<8, QT>(q0, q1, q2, q3, nu, cnu, btab, nv, Bp, Y, cf, lam4, err, st);
    case 16: return pj3_tc_go<16, QT>(q0, q1, q2, q3, nu, cnu, btab, nv, Bp, Y, cf, lam4, err, st);
    case 24: return pj3_tc_go<24, QT>(q0, q1, q2, q3, nu, cnu, btab, nv, Bp, Y, cf, lam4, err, st);
    default: return pj3_tc_go<32, QT>(q0, q1, q2, q3, nu, cnu, btab, nv, Bp, Y, cf, lam4, err, st);
    }
}

template cudaError_t launch_pj3_tc<float2>(const float2 *, const float2 *, const float2 *, const float2 *, double,
                                           const double *, const float *, int, int, int, float2 *, const float *,
                                           const double *, int *, cudaStream_t);
template cudaError_t launch_pj3_tc<double2>(const double2 *, const double2 *, const double2 *, const double2 *,
                                            double, const double *, const float *, int, int, int, float2 *,
                                            const float *, const double *, int *, cudaStream_t);

}  // namespace lp
