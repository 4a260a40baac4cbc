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
// split and stored by the block's 256 threads, two per row (each half of the
// row's k3 range, so twice the loads are in flight); one thread issues the
// 3 x (2n / 8) MMAs; the threads read back their rows of D (the two warps of
// a TMEM lane quarter taking alternate column chunks) and store Y
// cell-minor (each warp 32 consecutive cells, 256-byte stores).
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

constexpr int kThreads = 2 * kRows;  // two threads per row, each forming half of its K range

template <int N, typename QT>
__global__ void __launch_bounds__(kThreads) k_pj3_tc(const QT *__restrict__ q0, const QT *__restrict__ q1,
                                                     const QT *__restrict__ q2, const QT *__restrict__ q3, double nu,
                                                     const double *__restrict__ cnu, const float *__restrict__ btab,
                                                     int nv, int NP, int tcols, int Bp, float2 *__restrict__ Y,
                                                     const float *__restrict__ cf, const double *__restrict__ lam4,
                                                     int *__restrict__ err) {
    lp_grid_wait();
    constexpr int K = 2 * N, KC = K / 4;  // K of the real GEMM, its 16-byte core columns
    constexpr int NH = N / 2;             // k3 values per thread (a multiple of 4)
    extern __shared__ __align__(1024) unsigned char sm[];
    const uint32_t bbytes = (uint32_t)NP * K * 4;
    unsigned char *Bhi = sm, *Blo = sm + bbytes, *Ahi = sm + 2 * bbytes, *Alo = Ahi + kRows * K * 4;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, w = t >> 5, row = t & (kRows - 1), half = t >> 7;
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
    // this thread's half of its row: the RK4 combination along k3 in
    // [half * N/2, (half + 1) * N/2), loads issued four k3 at a time
    int pid, c;
    tile_row(blockIdx.x, row, Bp, pid, c);
    const double nuc = cnu ? cnu[c] : nu;
    const int kb = half * NH;
    float xr[NH], xi[NH];
    const long long b = ((long long)pid * N + kb) * Bp + c;
    if (cf) {
        constexpr int n3 = N * N * N;
        float l[4][5];
#pragma unroll
        for (int s = 0; s < 4; ++s)
#pragma unroll
            for (int j = 0; j < 5; ++j) l[s][j] = (float)lam4[(s * 5 + j) * Bp + c];
        const float nuf = (float)nuc;
#pragma unroll
        for (int k0 = 0; k0 < NH; k0 += 4) {
            QT qs[4][4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const long long o = b + (long long)(k0 + u) * Bp;
                qs[u][0] = q0[o]; qs[u][1] = q1[o]; qs[u][2] = q2[o]; qs[u][3] = q3[o];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int pt = pid * N + kb + k0 + u;
                const float r0 = cf[pt], r1 = cf[n3 + pt], r2 = cf[2 * n3 + pt], r3 = cf[3 * n3 + pt],
                            r4 = cf[4 * n3 + pt];
                float vr[4], vi[4];
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    vr[s] = (float)qs[u][s].x - (r0 * l[s][0] + r4 * l[s][4]);
                    vi[s] = (float)qs[u][s].y - (r1 * l[s][1] + r2 * l[s][2] + r3 * l[s][3]);
                }
                xr[k0 + u] = nuf * (0.5f * vr[0] + (vr[1] + vr[2] + vr[3]) * (1.f / 6.f));
                xi[k0 + u] = nuf * (0.5f * vi[0] + (vi[1] + vi[2] + vi[3]) * (1.f / 6.f));
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < NH; ++k) {
            const long long o = b + (long long)k * Bp;
            const QT a = q0[o], e = q1[o], d = q2[o], g = q3[o];
            xr[k] = (float)(nuc * (0.5 * a.x + (e.x + d.x + g.x) * (1. / 6.)));
            xi[k] = (float)(nuc * (0.5 * a.y + (e.y + d.y + g.y) * (1. / 6.)));
        }
    }
    // TF32 head and tail, 16 bytes (4 elements of K) per store
#pragma unroll
    for (int k = 0; k < NH; k += 4) {
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
        *reinterpret_cast<float4 *>(Ahi + tc::core_off(row, kb + k, KC)) = hr;
        *reinterpret_cast<float4 *>(Alo + tc::core_off(row, kb + k, KC)) = lr;
        *reinterpret_cast<float4 *>(Ahi + tc::core_off(row, N + kb + k, KC)) = hi4;
        *reinterpret_cast<float4 *>(Alo + tc::core_off(row, N + kb + k, KC)) = li4;
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
    bool done = tc::mbar_wait(&mbar[1], 0);
    if (!done) atomicExch(err, 2);
    done = __all_sync(0xffffffffu, done);  // the TMEM loads below are warp-wide
    tc::fence_after_sync();
    if (done) {
        // warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows), the two warps
        // of a lane quarter alternate 16-column chunks
        // column pair (a, j) of the chunk: one division per chunk, then the
        // output address advances by Bp per j and wraps to the next table
        const int ncol = 6 * nv;
        const uint32_t lane_base = tmem + ((uint32_t)(32 * (w & 3)) << 16);
        const long long awrap = (long long)N * N * nv * Bp - (long long)nv * Bp;
        for (int c0 = 16 * half; c0 < ncol; c0 += 32) {
            float v[16];
            tc::tmem_ld16(lane_base + (uint32_t)c0, v);
            const int aj0 = c0 >> 1, a0 = aj0 / nv;
            int j = aj0 - a0 * nv;
            long long o = (((long long)a0 * N * N + pid) * nv + j) * Bp + c;
#pragma unroll
            for (int u = 0; u < 16; u += 2) {
                if (c0 + u < ncol) Y[o] = make_float2(v[u], v[u + 1]);
                o += Bp;
                if (++j == nv) {
                    j = 0;
                    o += awrap;
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (w == 0) tc::tmem_free(tmem, (uint32_t)tcols);
}

// ---------------------------------------------------------------- axis 1
// The last pass of the projection (the CUDA-core version is k_pj1): per
// (pencil (j2, j3), cell) the five sources Z0..Z4 along k1 give, for every
// output j1, the real parts
//   a0 = Re T0 Z0, a1 = Re T1 Z0, a4 = Re T2 Z0 + Re T0 Z2 + Re T0 Z4,
//   a2 = Re T0 Z1, a3 = Re T0 Z3,
// then the increments d0..d4 of the record (j1, j2, j3) and the moment
// partials.  Re T z = sum_k Tr(k, j) Re z(k) - Ti(k, j) Im z(k) is a real
// GEMM with A = [Re z | Im z] per source and the shared operand
// [Tr; -Ti] per (table, j1): five K = 2n GEMMs per tile accumulate into
// TMEM columns [a0 | a1 | a4 | a2 | a3] (each block nvp = nv rounded up to
// 16 columns), the Z2 and Z4 products onto the a4 block.  The sources pass
// through one shared-memory A tile in turn: a source's rows are loaded into
// registers while the previous source's MMAs run.  A tile holds 128 rows:
// CBK = 64 cells (Bp a multiple of 64) or 32 of 2 or 4 pencils, so both
// pencils of a pair (j2, j3) = 2i, 2i + 1 are in the tile and the moment
// partial of (pair, cell) -- the layout k_lambda_inc reads -- is summed here.
struct PjMom {
    double dv12, dv6, dv2q, c19;
};

template <int N>
__global__ void __launch_bounds__(kThreads) k_pj1_tc(const float2 *__restrict__ Z, const float *__restrict__ btab,
                                                     int nv, int nvp, int Bp, int B, double dt, double kfac,
                                                     const double *__restrict__ cdt, double dv, double lv, PjMom mr,
                                                     float *__restrict__ Inc, double *__restrict__ part,
                                                     int *__restrict__ err) {
    lp_grid_wait();
    constexpr int K = 2 * N, KC = K / 4, NH = N / 2;
    extern __shared__ __align__(1024) unsigned char sm[];
    const uint32_t bbytes = (uint32_t)3 * nvp * K * 4;
    unsigned char *Bhi = sm, *Blo = sm + bbytes, *Ahi = sm + 2 * bbytes, *Alo = Ahi + kRows * K * 4;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tslot;
    __shared__ double red[5][kThreads];
    const int t = threadIdx.x, w = t >> 5, row = t & (kRows - 1), half = t >> 7;
    if (t == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (w == 0) tc::tmem_alloc(&tslot, 256u);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;
    if (t == 0) {
        tc::mbar_expect_tx(&mbar[0], 2 * bbytes);
        tc::bulk_g2s(Bhi, btab, 2 * bbytes, &mbar[0]);
    }
    const int CBK = (Bp % 64 == 0) ? 64 : 32, PP = kRows / CBK, ncb = Bp / CBK;
    const int g = blockIdx.x / ncb, cb = blockIdx.x - g * ncb;
    const int pq = g * PP + row / CBK, c = cb * CBK + (row % CBK);
    const long long zs = (long long)N * nv * nv * Bp, ks = (long long)nv * nv * Bp;
    const float2 *zrow = Z + (long long)(half * NH) * ks + (long long)pq * Bp + c;
    bool ok = true, have_b = true;  // have_b: thread 0 saw the shared operand arrive
    // the five sources in the order Z0, Z1, Z2, Z3, Z4
    for (int p = 0; p < 5; ++p) {
        float2 z[NH];
#pragma unroll
        for (int k = 0; k < NH; ++k) z[k] = zrow[p * zs + (long long)k * ks];
        if (p > 0 && !tc::mbar_wait(&mbar[1], (uint32_t)((p - 1) & 1))) {  // the A tile is free again
            ok = false;
            atomicExch(err, 2);
        }
#pragma unroll
        for (int k = 0; k < NH; k += 4) {
            float4 hr, lr, hi4, li4;
            float *phr = &hr.x, *plr = &lr.x, *phi = &hi4.x, *pli = &li4.x;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                phr[u] = tc::tf32_rna(z[k + u].x);
                plr[u] = tc::tf32_rna(z[k + u].x - phr[u]);
                phi[u] = tc::tf32_rna(z[k + u].y);
                pli[u] = tc::tf32_rna(z[k + u].y - phi[u]);
            }
            const int kk = half * NH + k;
            *reinterpret_cast<float4 *>(Ahi + tc::core_off(row, kk, KC)) = hr;
            *reinterpret_cast<float4 *>(Alo + tc::core_off(row, kk, KC)) = lr;
            *reinterpret_cast<float4 *>(Ahi + tc::core_off(row, N + kk, KC)) = hi4;
            *reinterpret_cast<float4 *>(Alo + tc::core_off(row, N + kk, KC)) = li4;
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (t == 0) {
            if (p == 0 && !tc::mbar_wait(&mbar[0], 0)) {
                have_b = false;
                atomicExch(err, 1);
                tc::mbar_wait(&mbar[0], 0);  // another bounded wait for the bulk copy before going on
            }
            if (have_b) {
                // destination block and width of this source: Z0 -> [a0 | a1 | a4]
                // (3 nvp columns), Z1 -> a2, Z3 -> a3, Z2 and Z4 -> onto a4
                const int col = p == 0 ? 0 : (p == 1 ? 3 * nvp : (p == 3 ? 4 * nvp : 2 * nvp));
                const int width = p == 0 ? 3 * nvp : nvp;
                const bool fresh = (p == 0 || p == 1 || p == 3);  // first products of these columns
                const uint32_t idesc = tc::idesc_tf32(kRows, width);
                const uint32_t lbo = 128, sbo = KC * 128;
                const unsigned char *As[3] = {Ahi, Ahi, Alo}, *Bs[3] = {Bhi, Blo, Bhi};
#pragma unroll
                for (int q = 0; q < 3; ++q)
#pragma unroll
                    for (int kq = 0; kq < K / 8; ++kq)
                        tc::mma_tf32(tmem + (uint32_t)col, tc::sdesc(tc::smem_u32(As[q]) + kq * 256, lbo, sbo),
                                     tc::sdesc(tc::smem_u32(Bs[q]) + kq * 256, lbo, sbo), idesc,
                                     !(fresh && q == 0 && kq == 0));
            }
            tc::mma_commit(&mbar[1]);  // completes phase p
        }
    }
    if (!tc::mbar_wait(&mbar[1], 0u)) {  // phase 4: every product is in TMEM
        ok = false;
        atomicExch(err, 2);
    }
    tc::fence_after_sync();
    // epilogue: this thread's row and j1 in [16 half, 16 half + 16).  The
    // TMEM loads are warp-wide (.sync.aligned): every lane of a warp takes
    // them or none does (j0 and the warp's agreement on `ok` are uniform;
    // whether a lane's cell is a padding cell is not)
    double m[5] = {0, 0, 0, 0, 0};
    const int j0 = 16 * half;
    ok = __all_sync(0xffffffffu, ok);
    if (ok && j0 < nv) {
        const uint32_t lane_base = tmem + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)j0;
        float a0[16], a1[16], a4[16], a2[16], a3[16];
        tc::tmem_ld16(lane_base, a0);
        tc::tmem_ld16(lane_base + (uint32_t)nvp, a1);
        tc::tmem_ld16(lane_base + (uint32_t)(2 * nvp), a4);
        tc::tmem_ld16(lane_base + (uint32_t)(3 * nvp), a2);
        tc::tmem_ld16(lane_base + (uint32_t)(4 * nvp), a3);
      if (c < B) {
        const int j2 = pq / nv, j3 = pq - j2 * nv;
        const float sf = (float)((cdt ? cdt[c] : dt) * kfac);
        DFSum S[5], T0, T1, T4, V0, V4;
#pragma unroll
        for (int jj = 0; jj < 16; ++jj) {
            const int j1 = j0 + jj;
            if (j1 >= nv) break;
            const float tp5 = a4[jj];
            const float d0 = sf * (4.75f * a0[jj] - 15.f * tp5), d4 = sf * (60.f * tp5 - 15.f * a0[jj]);
            const float d1 = 12.f * sf * a1[jj], d2 = 12.f * sf * a2[jj], d3 = 12.f * sf * a3[jj];
            const long long kt = ((long long)j1 * nv + j2) * nv + j3;
            float *o = Inc + kt * 5 * Bp + c;
            o[0] = d0; o[Bp] = d1; o[2 * Bp] = d2; o[3 * Bp] = d3; o[4 * Bp] = d4;
            S[0].add(d0); S[1].add(d1); S[2].add(d2); S[3].add(d3); S[4].add(d4);
            const float w1 = (float)jj, w2 = (float)(jj * jj);
            T0.addw(w1, d0); T1.addw(w1, d1); T4.addw(w1, d4);
            V0.addw(w2, d0); V4.addw(w2, d4);
        }
        const double G2 = -lv + (j2 + 0.5) * dv, G3 = -lv + (j3 + 0.5) * dv;
        const double G10 = -lv + (j0 + 0.5) * dv, G100 = G10 * G10, dv2 = dv * dv;
        const double S0 = S[0].get(), S1 = S[1].get(), S4 = S[4].get(), T0d = T0.get(), T1d = T1.get(),
                     T4d = T4.get();
        const double A0 = G10 * S0 + dv * T0d, A1 = G10 * S1 + dv * T1d, A4 = G10 * S4 + dv * T4d;
        const double B0 = G100 * S0 + 2. * G10 * dv * T0d + dv2 * V0.get();
        const double B4 = G100 * S4 + 2. * G10 * dv * T4d + dv2 * V4.get();
        const double S2 = S[2].get(), S3 = S[3].get();
        const double S04 = S0 + 0.25 * S4, G2233 = G2 * G2 + G3 * G3;
        m[0] = S04;
        m[1] = A0 + mr.dv12 * S1 + 0.25 * A4;
        m[2] = G2 * S04 + mr.dv12 * S2;
        m[3] = G3 * S04 + mr.dv12 * S3;
        m[4] = B0 + (G2233 + mr.dv2q) * S0 + mr.dv6 * (A1 + G2 * S2 + G3 * S3) + mr.c19 * S4 + 0.25 * B4 +
               0.25 * G2233 * S4;
      }
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) red[q][t] = m[q];
    tc::fence_before_sync();
    __syncthreads();
    // the moment partial of every (pencil pair, cell) of the tile: its two
    // pencils' rows, both halves of each, in a fixed order
    if (t < (PP / 2) * CBK) {
        const int pp = t / CBK, cc = t - pp * CBK;
        const int r0 = 2 * pp * CBK + cc, r1 = r0 + CBK;
        const int cell = cb * CBK + cc, pair = (g * PP) / 2 + pp, nblk = (nv * nv + 1) / 2;
        for (int q = 0; q < 5; ++q)
            part[((long long)cell * 5 + q) * nblk + pair] =
                ((red[q][r0] + red[q][r0 + kRows]) + red[q][r1]) + red[q][r1 + kRows];
    }
    __syncthreads();
    if (w == 0) tc::tmem_free(tmem, 256u);
}

// ---------------------------------------------------------------- axis 2
// The middle pass (the CUDA-core version is k_pj2): per (pencil (k1, j3),
// cell) the sources Y0, Y1, Y2 along k2 give Z_p(j2) = sum_k2 T_f(k2, j2)
// Y_a(k2) for (a, f) = (0, 0), (0, 1), (0, 2), (1, 0), (2, 0), p = 0..4 --
// complex GEMMs with the axis-3 pass's shared operand (its first 2 nv
// columns are T0's): Y0 times all 6 nv columns into TMEM [Z0 | Z1 | Z2], Y1
// and Y2 times T0's 2 nv columns into [Z3], [Z4] (10 nv <= 256 columns).
// The sources pass through one A tile in turn, as in the axis-1 pass.
template <int N>
__global__ void __launch_bounds__(kThreads) k_pj2_tc(const float2 *__restrict__ Y, const float *__restrict__ btab,
                                                     int nv, int Bp, float2 *__restrict__ Z, int *__restrict__ err) {
    lp_grid_wait();
    constexpr int K = 2 * N, KC = K / 4, NH = N / 2;
    extern __shared__ __align__(1024) unsigned char sm[];
    const uint32_t bbytes = (uint32_t)6 * nv * K * 4;
    unsigned char *Bhi = sm, *Blo = sm + bbytes, *Ahi = sm + 2 * bbytes, *Alo = Ahi + kRows * K * 4;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tslot;
    const int t = threadIdx.x, w = t >> 5, row = t & (kRows - 1), half = t >> 7;
    if (t == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    if (w == 0) tc::tmem_alloc(&tslot, 256u);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tslot;
    if (t == 0) {
        tc::mbar_expect_tx(&mbar[0], 2 * bbytes);
        tc::bulk_g2s(Bhi, btab, 2 * bbytes, &mbar[0]);
    }
    int pen, c;
    tile_row(blockIdx.x, row, Bp, pen, c);
    const int k1 = pen / nv, j3 = pen - k1 * nv;
    const long long ys = (long long)N * N * nv * Bp, kstride = (long long)nv * Bp;
    const float2 *yrow = Y + (((long long)k1 * N + half * NH) * nv + j3) * Bp + c;
    bool ok = true, have_b = true;
    for (int a = 0; a < 3; ++a) {
        float2 y[NH];
#pragma unroll
        for (int k = 0; k < NH; ++k) y[k] = yrow[a * ys + (long long)k * kstride];
        if (a > 0 && !tc::mbar_wait(&mbar[1], (uint32_t)((a - 1) & 1))) {
            ok = false;
            atomicExch(err, 2);
        }
#pragma unroll
        for (int k = 0; k < NH; k += 4) {
            float4 hr, lr, hi4, li4;
            float *phr = &hr.x, *plr = &lr.x, *phi = &hi4.x, *pli = &li4.x;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                phr[u] = tc::tf32_rna(y[k + u].x);
                plr[u] = tc::tf32_rna(y[k + u].x - phr[u]);
                phi[u] = tc::tf32_rna(y[k + u].y);
                pli[u] = tc::tf32_rna(y[k + u].y - phi[u]);
            }
            const int kk = half * NH + k;
            *reinterpret_cast<float4 *>(Ahi + tc::core_off(row, kk, KC)) = hr;
            *reinterpret_cast<float4 *>(Alo + tc::core_off(row, kk, KC)) = lr;
            *reinterpret_cast<float4 *>(Ahi + tc::core_off(row, N + kk, KC)) = hi4;
            *reinterpret_cast<float4 *>(Alo + tc::core_off(row, N + kk, KC)) = li4;
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (t == 0) {
            if (a == 0 && !tc::mbar_wait(&mbar[0], 0)) {
                have_b = false;
                atomicExch(err, 1);
                tc::mbar_wait(&mbar[0], 0);  // another bounded wait for the bulk copy before going on
            }
            if (have_b) {
                const int col = a == 0 ? 0 : (a == 1 ? 6 * nv : 8 * nv);
                const int width = a == 0 ? 6 * nv : 2 * nv;
                const uint32_t idesc = tc::idesc_tf32(kRows, width);
                const uint32_t lbo = 128, sbo = KC * 128;
                const unsigned char *As[3] = {Ahi, Ahi, Alo}, *Bs[3] = {Bhi, Blo, Bhi};
#pragma unroll
                for (int q = 0; q < 3; ++q)
#pragma unroll
                    for (int kq = 0; kq < K / 8; ++kq)
                        tc::mma_tf32(tmem + (uint32_t)col, tc::sdesc(tc::smem_u32(As[q]) + kq * 256, lbo, sbo),
                                     tc::sdesc(tc::smem_u32(Bs[q]) + kq * 256, lbo, sbo), idesc, q > 0 || kq > 0);
            }
            tc::mma_commit(&mbar[1]);  // completes phase a
        }
    }
    if (!tc::mbar_wait(&mbar[1], 0u)) {  // phase 2: every product is in TMEM
        ok = false;
        atomicExch(err, 2);
    }
    ok = __all_sync(0xffffffffu, ok);  // the TMEM loads below are warp-wide
    tc::fence_after_sync();
    if (ok) {
        // columns (p, j2, re/im) of this thread's row; the two warps of a lane
        // quarter take alternate 16-column chunks
        // column pair (p, j2) of the chunk: one division per chunk, then the
        // output address advances by nv Bp per j2 and wraps to the next source
        const long long zs = (long long)N * nv * nv * Bp, js = (long long)nv * Bp;
        const int ncol = 10 * nv;
        const uint32_t lane_base = tmem + ((uint32_t)(32 * (w & 3)) << 16);
        for (int c0 = 16 * half; c0 < ncol; c0 += 32) {
            float v[16];
            tc::tmem_ld16(lane_base + (uint32_t)c0, v);
            const int pj0 = c0 >> 1, p0 = pj0 / nv;
            int j2 = pj0 - p0 * nv;
            long long o = p0 * zs + (((long long)k1 * nv + j2) * nv + j3) * Bp + c;
#pragma unroll
            for (int u = 0; u < 16; u += 2) {
                if (c0 + u < ncol) Z[o] = make_float2(v[u], v[u + 1]);
                o += js;
                if (++j2 == nv) {
                    j2 = 0;
                    o += zs - (long long)nv * js;
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (w == 0) tc::tmem_free(tmem, 256u);
}

}  // namespace

bool pj2_tc_supported(int n, int nv, int Bp) {
    if (!(n == 8 || n == 16 || n == 24 || n == 32)) return false;
    if (nv < 8 || nv % 8 || 10 * nv > 256) return false;  // 2 nv and 6 nv multiples of 16
    if (Bp < 32 || Bp % 32) return false;
    return ((long long)n * nv * Bp) % kRows == 0;
}

size_t pj2_tc_smem(int n, int nv) { return (size_t)2 * 6 * nv * 2 * n * 4 + (size_t)2 * kRows * 2 * n * 4; }

int pj1_tc_nvp(int nv) { return ((nv + 15) / 16) * 16; }

bool pj1_tc_supported(int n, int nv, int Bp) {
    if (!(n == 8 || n == 16 || n == 24 || n == 32)) return false;
    if (nv < 2 || nv > 32 || (nv & 1)) return false;
    return Bp >= 32 && Bp % 32 == 0;
}

size_t pj1_tc_table_floats(int n, int nv) { return (size_t)2 * 3 * pj1_tc_nvp(nv) * 2 * n; }

size_t pj1_tc_smem(int n, int nv) { return pj1_tc_table_floats(n, nv) * 4 + (size_t)2 * kRows * 2 * n * 4; }

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
    k_pj3_tc<N, QT><<<tiles, kThreads, smem, st>>>(q0, q1, q2, q3, nu, cnu, btab, nv, NP, tcols, Bp, Y, cf, lam4,
                                                    err);
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


// The shared operand of the axis-1 pass: rows (table a, output j1) = the
// real-part column [Tr(., j1); -Ti(., j1)] of T0, T1, T2, each table padded
// to nvp rows, TF32 head then tail, in the MMA's shared-memory layout.
void pj1_tc_table(const float *tfac, int n, int nv, std::vector<float> &out) {
    const int K = 2 * n, KC = K / 4, nvp = pj1_tc_nvp(nv);
    out.assign(pj1_tc_table_floats(n, nv), 0.f);
    float *hi = out.data(), *lo = out.data() + (size_t)3 * nvp * K;
    for (int a = 0; a < 3; ++a)
        for (int j = 0; j < nv; ++j)
            for (int k = 0; k < n; ++k) {
                const size_t t = ((size_t)a * n + k) * nv + j;
                const float vals[2] = {tfac[2 * t], -tfac[2 * t + 1]};
                for (int e = 0; e < 2; ++e) {
                    const float h = tf32_round_host(vals[e]);
                    const float l = tf32_round_host(vals[e] - h);
                    const int off = tc::core_off(a * nvp + j, e * n + k, KC) / 4;
                    hi[off] = h;
                    lo[off] = l;
                }
            }
}

template <int N>
static cudaError_t pj1_tc_go(const float2 *Z, const float *btab, int nv, int Bp, int B, double dt, double kfac,
                             const double *cdt, double dv, double lv, float *Inc, double *part, int *err,
                             cudaStream_t st) {
    const size_t smem = pj1_tc_smem(N, nv);
    cudaError_t e = cudaFuncSetAttribute(k_pj1_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int CBK = (Bp % 64 == 0) ? 64 : 32, PP = kRows / CBK;
    const int tiles = (nv * nv / PP) * (Bp / CBK);
    const PjMom mr{dv / 12., dv / 6., dv * dv / 4., 19. * dv * dv / 240.};
    k_pj1_tc<N><<<tiles, kThreads, smem, st>>>(Z, btab, nv, pj1_tc_nvp(nv), Bp, B, dt, kfac, cdt, dv, lv, mr, Inc,
                                               part, err);
    return cudaGetLastError();
}

cudaError_t launch_pj1_tc(const float2 *Z, const float *btab, int n, int nv, int Bp, int B, double dt, double kfac,
                          const double *cdt, double dv, double lv, float *Inc, double *part, int *err,
                          cudaStream_t st) {
    if (!pj1_tc_supported(n, nv, Bp) || !btab || !err) return cudaErrorInvalidValue;
    const int PP = kRows / ((Bp % 64 == 0) ? 64 : 32);
    if ((nv * nv) % PP) return cudaErrorInvalidValue;
    if (reinterpret_cast<uintptr_t>(btab) % 16) return cudaErrorInvalidValue;
    switch (n) {
    case 8: return pj1_tc_go<8>(Z, btab, nv, Bp, B, dt, kfac, cdt, dv, lv, Inc, part, err, st);
    case 16: return pj1_tc_go<16>(Z, btab, nv, Bp, B, dt, kfac, cdt, dv, lv, Inc, part, err, st);
    case 24: return pj1_tc_go<24>(Z, btab, nv, Bp, B, dt, kfac, cdt, dv, lv, Inc, part, err, st);
    default: return pj1_tc_go<32>(Z, btab, nv, Bp, B, dt, kfac, cdt, dv, lv, Inc, part, err, st);
    }
}


template <int N>
static cudaError_t pj2_tc_go(const float2 *Y, const float *btab, int nv, int Bp, float2 *Z, int *err,
                             cudaStream_t st) {
    const size_t smem = pj2_tc_smem(N, nv);
    cudaError_t e = cudaFuncSetAttribute(k_pj2_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int tiles = (int)((long long)N * nv * Bp / kRows);
    k_pj2_tc<N><<<tiles, kThreads, smem, st>>>(Y, btab, nv, Bp, Z, err);
    return cudaGetLastError();
}

cudaError_t launch_pj2_tc(const float2 *Y, const float *btab, int n, int nv, int Bp, float2 *Z, int *err,
                          cudaStream_t st) {
    if (!pj2_tc_supported(n, nv, Bp) || !btab || !err) return cudaErrorInvalidValue;
    if (pj3_tc_np(nv) != 6 * nv) return cudaErrorInvalidValue;  // the axis-3 table without padding columns
    if (reinterpret_cast<uintptr_t>(btab) % 16) return cudaErrorInvalidValue;
    switch (n) {
    case 8: return pj2_tc_go<8>(Y, btab, nv, Bp, Z, err, st);
    case 16: return pj2_tc_go<16>(Y, btab, nv, Bp, Z, err, st);
    case 24: return pj2_tc_go<24>(Y, btab, nv, Bp, Z, err, st);
    default: return pj2_tc_go<32>(Y, btab, nv, Bp, Z, err, st);
    }
}

}  // namespace lp
