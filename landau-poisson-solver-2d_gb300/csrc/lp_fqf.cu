// ComputeQ's convolution form (the seven windowed convolutions of
// lp_fftq.cu) with the axis-2 spectra kept on chip.
//
// The three-pass form writes the axis-2 spectra X of the 13 arrays (7 a-,
// 6 b-arrays: 13 n M^2 complex values per cell) to DRAM and reads them
// straight back for the direct sums along axis 1.  Here:
//
//   k_fq_x1   axis-3 DFTs of the 10 source arrays (the 7 a-arrays C_p F and
//             F (u3 - h)^e3, e3 = 0, 1, 2) into X1 (10 n^2 M per cell: a
//             little over half of X), blocked so that the n x n values of
//             one (cell group, k3, array) form one contiguous slice;
//   k_fq_yz   per (k3, group of CB cells): the axis-2 DFTs of the pair's two
//             arrays from their X1 slices, the direct sums along axis 1 over
//             the seven pairs, and the inverse axis-2 DFT of the n kept
//             outputs, into H (the input of the inverse axis-3 pass, which
//             is shared with the three-pass form).
//
// k_fq_yz is persistent (one CTA per SM takes tile after tile) and runs a
// producer / consumer pipeline over the seven pairs of its tiles.  One
// producer thread brings a pair's two X1 slices into shared memory with
// cp.async.bulk (two slots, so the pair two steps ahead streams in while
// this one is transformed); the producer warps transform them along axis 2
// into one of two spectrum slots; the consumer warps (one thread per (k2,
// cell, output parity)) sum the slot along axis 1 while the producers fill
// the other slot, and after a tile's seventh pair run its inverse axis-2
// DFTs while the producers start on the next tile.  The hand-offs are
// mbarriers: fa and fb (the a- and b-slice bulk copies landed), full2
// (spectra written), empty2 (spectra read).  Every wait is bounded in time; a wait that runs out sets
// *err and that thread waits no more, so the kernel ends.
//
// The arithmetic is that of the three-pass form except for where the
// axis-1 weight (u1 - h)^e1 of the b-arrays enters: here it scales the
// b-pencil before its axis-2 DFT (an exact integer factor combined with
// (u2 - h)^e2), there the axis-2 outputs during the axis-1 sum.  Both forms
// agree to FP32 rounding.
#include "lp_kernels.cuh"
#include "lp_dev.cuh"
#include "lp_fft.cuh"
#include "lp_tc.cuh"

namespace lp {
namespace {

// Cells per tile (CB) and producer warps (PW) per n.
template <int N> struct FqfCfg;
template <> struct FqfCfg<8> { static constexpr int CB = 16, PW = 8; };  // PW = 2 N CB / 32
template <> struct FqfCfg<16> { static constexpr int CB = 4, PW = 4; };
template <> struct FqfCfg<24> { static constexpr int CB = 4, PW = 6; };
template <> struct FqfCfg<32> { static constexpr int CB = 2, PW = 4; };

template <int N> struct Fqf {
    static constexpr int M = 3 * N / 2;
    static constexpr int CB = FqfCfg<N>::CB, PW = FqfCfg<N>::PW;
    // Rows (one per axis-1 index l) of an X1 slice [l][m][cell] and of a
    // spectrum [l][k2][cell], padded by one cell group when CB < 16: the
    // threads of a half-warp then read (and write) rows that start in
    // different banks.
    static constexpr int RS1 = CB < 16 ? (N + 1) * CB : N * CB;
    static constexpr int SL1 = N * RS1;  // one X1 slice (float2)
    static constexpr int RS2 = CB < 16 ? (M + 1) * CB : M * CB;
    static constexpr int SL2 = N * RS2;  // one array's spectrum in shared memory
    // consumer threads: two (the real and imaginary parts of the a-arrays)
    // per (k2, cell) of a tile;
    // producer threads after them
    static constexpr int UY = M * CB, TY = 2 * UY, TP = 32 * PW, T = TY + TP;
    // two a-slice slots, two b-slice slots, two spectrum slots of a pair's
    // two arrays and a tile's axis-1 sums G
    static constexpr size_t smem = sizeof(float2) * (4 * (size_t)SL1 + 5 * (size_t)SL2);
    static_assert(TY % 32 == 0 && (N * CB) % 32 == 0, "warps of one role; pencil tasks of a warp share their array");
    static_assert(2 * N * CB == TP, "one pencil task per producer thread and pair");
    static_assert((SL1 * sizeof(float2)) % 16 == 0, "bulk copies move multiples of 16 bytes");
};

// The pairs: a-array p (X1 array p) with the b-array formed from X1 array
// bsrc(p) = 7 + e3 times (u2 - h)^e2 (u1 - h)^e1 before the axis-2 DFT.  (ahat, 1), (S00, u1^2), (S11, u2^2),
// (S22, u3^2), (S01, u1 u2), (S02, u1 u3), (S12, u2 u3).
__device__ __forceinline__ int bsrc(int p) { return p == 3 ? 9 : (p >= 5 ? 8 : 7); }
__device__ __forceinline__ int be2(int p) { return p == 2 ? 2 : ((p == 4 || p == 6) ? 1 : 0); }
__device__ __forceinline__ int be1(int p) { return p == 1 ? 2 : ((p == 4 || p == 5) ? 1 : 0); }
// The b-slice of pair p changes at p = 0, 3, 4, 5 (X1 arrays 7, 9, 7, 8):
// the pairs' b-slice events 0 (p 0..2), 1 (p 3), 2 (p 4), 3 (p 5, 6).
__device__ __forceinline__ int bev(int p) { return p < 3 ? 0 : (p < 5 ? p - 2 : 3); }
__device__ __forceinline__ bool bstart(int p) { return p == 0 || p == 3 || p == 4 || p == 5; }

// Axis-3 DFTs: one thread per (array, l, m, cell) pencil, the M outputs
// stored at X1[((group * M + k3) * 10 + array) * SL1 + l * RS1 + m * CB + cc]
// (group = cell / CB, cc = cell % CB).  The 32 lanes of a warp take
// consecutive (m, cc), so the stores of one k3 are contiguous.
template <int N>
__global__ void __launch_bounds__(128) k_fq_x1(const float2 *__restrict__ F, const float *__restrict__ C, int Bp,
                                               int c0, int Bc, float2 *__restrict__ X1, FftTw tw) {
    lp_grid_wait();
    using P = Fqf<N>;
    constexpr int n = N, h = N / 2, CB = P::CB;
    const long long g = (long long)blockIdx.x * 128 + threadIdx.x;
    if (g >= 10LL * n * n * Bc) return;
    const int cc = (int)(g % CB);
    const long long r = g / CB;
    const int lm = (int)(r % (n * n));
    const int r2 = (int)(r / (n * n));
    const int arr = r2 % 10, cgp = r2 / 10;
    const int l = lm / n, m = lm - l * n;
    const float2 *src = F + (size_t)lm * n * Bp + c0 + cgp * CB + cc;
    float2 *dst = X1 + ((size_t)cgp * P::M * 10 + arr) * P::SL1 + l * P::RS1 + m * CB + cc;
    constexpr size_t ks = (size_t)10 * P::SL1;  // stride of k3
    auto st = [&](int k, float2 v) { dst[k * ks] = v; };
    float2 x[N];
    if (arr < 7) {
        // the pencil's n weights are contiguous and 16-byte aligned (n a
        // multiple of 4, C from cudaMalloc): n / 4 vector loads
        const float4 *cp = reinterpret_cast<const float4 *>(C + (size_t)arr * n * n * n + (size_t)lm * n);
#pragma unroll
        for (int q4 = 0; q4 < n / 4; ++q4) {
            const float4 w = __ldg(cp + q4);
            x[4 * q4] = cscale(src[(size_t)(4 * q4) * Bp], w.x);
            x[4 * q4 + 1] = cscale(src[(size_t)(4 * q4 + 1) * Bp], w.y);
            x[4 * q4 + 2] = cscale(src[(size_t)(4 * q4 + 2) * Bp], w.z);
            x[4 * q4 + 3] = cscale(src[(size_t)(4 * q4 + 3) * Bp], w.w);
        }
        fwd_pencil_st<N, true>(x, tw.fa, st);
    } else {
#pragma unroll
        for (int q = 0; q < n; ++q) x[q] = cscale(src[(size_t)q * Bp], poww(q, h, arr - 7));
        fwd_pencil_st<N, false>(x, tw.fw, st);
    }
}

// One pair's direct sum along axis 1 for every output i of one (k2, k3,
// cell), one component of a per thread: P[i] += a_s(l) (b.x, b.y)(u) with
// u = i + h - l, a_s = Re a (s = 0) or Im a (s = 1), a(l) and b(u) from the
// spectrum rows (stride RS), b already weighted by (u1 - h)^e1 (the
// producers fold that weight into the scaling of the b-pencil before its
// axis-2 DFT).  The two threads of a lane pair hold the two components; a
// b-row is held in registers, only the (i, l) with u on the grid are
// summed, and each output sums its terms in l ascending order.
template <int N, int RS>
__device__ __forceinline__ void ysum_c(const float2 *__restrict__ as, const float2 *__restrict__ bs, int s,
                                       unsigned long long (&P)[N]) {
    constexpr int n = N, h = N / 2;
    unsigned long long yb[N];
#pragma unroll
    for (int u = 0; u < n; ++u) {
        const float2 val = bs[u * RS];
        yb[u] = pk2(val.x, val.y);
    }
    const float *ac = reinterpret_cast<const float *>(as) + s;
#pragma unroll
    for (int l = 0; l < n; ++l) {
        const float a = ac[2 * l * RS];
        const unsigned long long a2 = pk2(a, a);
#pragma unroll
        for (int i = 0; i < n; ++i) {
            const int u = i + h - l;
            if (u >= 0 && u < n) P[i] = fma2(a2, yb[u], P[i]);
        }
    }
}

// a bounded wait; after one of this thread's waits ran out it waits no more
__device__ __forceinline__ void fq_wait(uint64_t *mb, uint32_t parity, int *err, bool &bad, int code) {
    if (bad) return;
    if (!tc::mbar_wait_susp(mb, parity)) {
        bad = true;
        if (err) atomicExch(err, code);
    }
}

// Persistent: CTA b takes the tiles (k3, cell group) t = b, b + grid, ...;
// its steps g = 7 i + p run over (its i-th tile, pair p), and the pipeline
// runs on across tiles (the next tile's first slices stream in while this
// tile's last pairs are summed; the consumers' inverse axis-2 DFTs of one
// tile overlap the producers' first pairs of the next).  (An L2 prefetch of
// the next tile's slices measured 5% slower: the copies' DRAM traffic is
// already one pass over X1.)
//
// Shared memory: a-slices in two slots (step g in slot g & 1), b-slices in
// two slots (b-slice event E = 4 i + bev(p) in slot E & 1: the b-slice is
// loaded only when it changes), both filled two steps ahead once every
// producer has transformed step g (the slots' previous contents have been
// read by then); spectra in two slots (step g in slot g & 1); G of a tile.
// mbarriers: fa[2] and fb[2] (bulk copies landed), full2[2] (spectra
// written by the producers), empty2[2] (spectra read by the consumers).
template <int N>
__global__ void __launch_bounds__(Fqf<N>::T, 1) k_fq_yz(const float2 *__restrict__ X1, int ntile, int Bs,
                                                         float2 *__restrict__ H, FftTw tw, int *__restrict__ err) {
    lp_grid_wait();
    using P = Fqf<N>;
    constexpr int n = N, h = N / 2, M = P::M, CB = P::CB, NJ = N / 2;
    extern __shared__ __align__(128) float2 fsm[];
    float2 *a1 = fsm;                // [2][SL1] a-slices
    float2 *b1 = fsm + 2 * P::SL1;   // [2][SL1] b-slices
    float2 *s2 = fsm + 4 * P::SL1;   // [slot][a, b][SL2] spectra
    float2 *gs = s2 + 4 * P::SL2;    // [i1][k2][cc] a tile's axis-1 sums
    __shared__ __align__(8) uint64_t bar[8];  // fa[2], fb[2], full2[2], empty2[2]
    // the axis-2 twiddles of the a-side (with the output phase) and of the
    // b-side: one DFT routine serves both through a table pointer (the
    // b-side's q2 = 0 row is exactly 1, so applying it changes nothing),
    // which halves the producers' unrolled code
    __shared__ float2 tws[2][48];
    uint64_t *fa = bar, *fb = bar + 2, *full2 = bar + 4, *empty2 = bar + 6;
    const int tid = threadIdx.x;
    if (tid < 48) {
        tws[0][tid] = tw.fa[tid];
        tws[1][tid] = tw.fw[tid];
    }
    const int my_tiles = (ntile - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    const int G = 7 * my_tiles;
    const bool issuer = tid == P::TY;
    constexpr uint32_t slice_bytes = P::SL1 * sizeof(float2);
    if (issuer) {
        for (int k = 0; k < 4; ++k) tc::mbar_init(&bar[k], 1);
        tc::mbar_init(&full2[0], P::TP);
        tc::mbar_init(&full2[1], P::TP);
        tc::mbar_init(&empty2[0], P::TY);
        tc::mbar_init(&empty2[1], P::TY);
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    __syncthreads();
    auto tile_base = [&](int i) {  // the ten X1 slices of this CTA's i-th tile
        const int t = (int)blockIdx.x + i * (int)gridDim.x, k3 = t % M, cgp = t / M;
        return X1 + ((size_t)cgp * M + k3) * 10 * P::SL1;
    };
    auto afill = [&](int g) {  // step g's a-slice into slot g & 1
        const int sa = g & 1, p = g % 7, i = g / 7;
        tc::fence_async_smem();
        tc::mbar_expect_tx(&fa[sa], slice_bytes);
        tc::bulk_g2s(a1 + sa * P::SL1, tile_base(i) + (size_t)p * P::SL1, slice_bytes, &fa[sa]);
    };
    auto bfill = [&](int g) {  // the b-slice event starting at step g into its slot
        const int p = g % 7, i = g / 7, sb = (4 * i + bev(p)) & 1;
        tc::fence_async_smem();
        tc::mbar_expect_tx(&fb[sb], slice_bytes);
        tc::bulk_g2s(b1 + sb * P::SL1, tile_base(i) + (size_t)bsrc(p) * P::SL1, slice_bytes, &fb[sb]);
    };
    if (issuer) {
        for (int g = 0; g < 2 && g < G; ++g) afill(g);
        bfill(0);
    }
    bool bad = false;
    if (tid >= P::TY) {
        // producers: the axis-2 DFT of one (array, l, cell) pencil of the
        // pair per thread, the warps' pencils sharing their array
        const int tp = tid - P::TY;
        const int cc = tp % CB, l = (tp / CB) % n, which = tp / (n * CB);
        for (int g = 0; g < G; ++g) {
            const int s = g & 1, p = g % 7, e2 = be2(p), E = 4 * (g / 7) + bev(p);
            fq_wait(&fa[s], (uint32_t)((g >> 1) & 1), err, bad, 3);
            fq_wait(&fb[E & 1], (uint32_t)((E >> 1) & 1), err, bad, 3);
            float2 x[N];
            {
                const float2 *src = (which ? b1 + (E & 1) * P::SL1 : a1 + s * P::SL1) + l * P::RS1 + cc;
#pragma unroll
                for (int m = 0; m < n; ++m) x[m] = src[m * CB];
            }
            if (g >= 2) fq_wait(&empty2[s], (uint32_t)(((g - 2) >> 1) & 1), err, bad, 4);
            float2 *dst = s2 + (2 * s + which) * P::SL2 + l * P::RS2 + cc;
            auto st = [&](int k, float2 v) { dst[k * CB] = v; };
            if (which) {
                // (u2 - h)^e2 along the pencil times (u1 - h)^e1 of its row:
                // small integers, so the combined weight is exact in FP32
                const int e1 = be1(p);
                if (e2 || e1) {
                    const float w1 = poww(l, h, e1);
#pragma unroll
                    for (int m = 0; m < n; ++m) x[m] = cscale(x[m], poww(m, h, e2) * w1);
                }
            }
            fwd_pencil_st<N, true>(x, tws[which], st);
            tc::mbar_arrive(&full2[s]);
            // refills two steps ahead once every producer has read step g's slices
            tc::fence_async_smem();    // this thread's slice reads before the bulk copies' writes
            tc::named_sync(1, P::TP);
            if (issuer && g + 2 < G) {
                afill(g + 2);
                if (bstart((g + 2) % 7)) bfill(g + 2);
            }
        }
    } else {
        // consumers: the lane pair (k2, cc) sums every output of every pair
        // of its tile, lane s with component s of a (P0 = Re a b, P1 = Im a b,
        // G = (P0.x - P1.y, P0.y + P1.x)), then the tile's inverse axis-2 DFTs
        const int r = tid & 1, uid = tid >> 1, k2 = uid / CB, cc = uid % CB;
        for (int i = 0; i < my_tiles; ++i) {
            unsigned long long Pc[N];
#pragma unroll
            for (int j = 0; j < N; ++j) Pc[j] = 0ull;
            for (int p = 0; p < 7; ++p) {
                const int g = 7 * i + p, s = g & 1;
                fq_wait(&full2[s], (uint32_t)((g >> 1) & 1), err, bad, 5);
                const float2 *as = s2 + (2 * s) * P::SL2 + k2 * CB + cc, *bs = as + P::SL2;
                ysum_c<N, P::RS2>(as, bs, r, Pc);
                if (g + 2 < G) tc::mbar_arrive(&empty2[s]);
            }
            tc::named_sync(2, P::TY);  // the previous tile's inverse DFTs are done with gs
            {
                // lane r writes the outputs i = 2 j + r, taking the partner's
                // component of them in exchange for its own of the others
                float2 *gp = gs + r * P::RS2 + k2 * CB + cc;
#pragma unroll
                for (int j = 0; j < NJ; ++j) {
                    const float2 send = up2(r ? Pc[2 * j] : Pc[2 * j + 1]), own = up2(r ? Pc[2 * j + 1] : Pc[2 * j]);
                    const float2 got = make_float2(__shfl_xor_sync(0xffffffffu, send.x, 1),
                                                   __shfl_xor_sync(0xffffffffu, send.y, 1));
                    const float2 p0 = r ? got : own, p1 = r ? own : got;
                    gp[2 * j * P::RS2] = make_float2(p0.x - p1.y, p0.y + p1.x);
                }
            }
            tc::named_sync(2, P::TY);
            // inverse axis-2 DFT of the (i1, cell) pencils, outputs xi2 in
            // [0, n), into H[((i1 n + xi2) M + k3) Bs + cell]
            const int t = (int)blockIdx.x + i * (int)gridDim.x, k3 = t % M, cgp = t / M;
            for (int jt = tid; jt < n * CB; jt += P::TY) {
                const int c2 = jt % CB, i1 = jt / CB;
                const float2 *src = gs + i1 * P::RS2 + c2;
                float2 gv[M], x[N];
#pragma unroll
                for (int k = 0; k < M; ++k) gv[k] = src[k * CB];
                inv_pencil<N>(gv, x, tw.iv);
                float2 *dst = H + ((size_t)i1 * n * M + k3) * Bs + cgp * CB + c2;
#pragma unroll
                for (int j2 = 0; j2 < n; ++j2) dst[(size_t)j2 * M * Bs] = x[j2];
            }
        }
    }
}

template <int N>
cudaError_t launch_fused(const float2 *F, const float *C, const FftTw &tw, int Bp, int c0, int Bc, float2 *X1,
                         float2 *H, int Bs, cudaStream_t st, int stage, int *err) {
    using P = Fqf<N>;
    if (Bc % P::CB) return cudaErrorInvalidValue;
    if (stage < 0 || stage == 0) {
        const long long th = 10LL * N * N * Bc;
        k_fq_x1<N><<<(unsigned)((th + 127) / 128), 128, 0, st>>>(F, C, Bp, c0, Bc, X1, tw);
    }
    if (stage < 0 || stage == 2) {
        // opt-in above 48 KB of dynamic shared memory (per device, so on every call)
        cudaError_t e = cudaFuncSetAttribute(k_fq_yz<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P::smem);
        if (e != cudaSuccess) return e;
        // persistent: as many CTAs as fit on the device at once, at most one per tile
        int dev = 0, sms = 0, per_sm = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fq_yz<N>, P::T, P::smem)) != cudaSuccess)
            return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
        const int ntile = P::M * (Bc / P::CB);
        const int grid = ntile < sms * per_sm ? ntile : sms * per_sm;
        k_fq_yz<N><<<grid, P::T, P::smem, st>>>(X1, ntile, Bs, H, tw, err);
    }
    return cudaGetLastError();
}

}  // namespace

size_t fq_fused_x1_elems(int n, int Bs) {
    switch (n) {
    case 8: return (size_t)Bs / Fqf<8>::CB * Fqf<8>::M * 10 * Fqf<8>::SL1;
    case 16: return (size_t)Bs / Fqf<16>::CB * Fqf<16>::M * 10 * Fqf<16>::SL1;
    case 24: return (size_t)Bs / Fqf<24>::CB * Fqf<24>::M * 10 * Fqf<24>::SL1;
    case 32: return (size_t)Bs / Fqf<32>::CB * Fqf<32>::M * 10 * Fqf<32>::SL1;
    default: return 0;
    }
}

cudaError_t launch_fq_fused(int n, const float2 *F, const float *C, const FftTw &tw, int Bp, int c0, int Bc,
                            float2 *X1, float2 *H, int Bs, cudaStream_t st, int stage, int *err) {
    switch (n) {
    case 8: return launch_fused<8>(F, C, tw, Bp, c0, Bc, X1, H, Bs, st, stage, err);
    case 16: return launch_fused<16>(F, C, tw, Bp, c0, Bc, X1, H, Bs, st, stage, err);
    case 24: return launch_fused<24>(F, C, tw, Bp, c0, Bc, X1, H, Bs, st, stage, err);
    case 32: return launch_fused<32>(F, C, tw, Bp, c0, Bc, X1, H, Bs, st, stage, err);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace lp
