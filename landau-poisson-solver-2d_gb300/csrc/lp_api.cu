// Context and C ABI of the GB300 Landau-Poisson hot path (include/lp_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "lp_gb300.h"
#include "lp_adjoint.cuh"
#include "lp_kernels.cuh"
#include "lp_tables.h"

using lp::V2;

// An NVTX range over a host scope: the stages of a step appear as named
// ranges in Nsight timelines and ncu's NVTX filters (no cost without a tool
// attached).  Work that a CUDA graph replays is marked where it is captured
// and where the graph is launched.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

constexpr int kHostChunksMax = 16;  // chunks of lp_collision_step_host

struct lp_ctx {
    lp::Tables T;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    std::string err;
    size_t bytes = 0;
    std::vector<void *> allocs;
    bool mixed = false;
    // tables
    double *eta = nullptr, *shat = nullptr, *ahat = nullptr, *cw = nullptr, *c1 = nullptr, *c2 = nullptr,
           *cct = nullptr, *nodeoff = nullptr;
    unsigned char *rzero = nullptr, *gate = nullptr;
    int *nodecell = nullptr, *pair_off = nullptr, *ipiv = nullptr;
    void *tfac = nullptr, *mfwd = nullptr, *minv = nullptr;  // R precision
    // the FP32 per-axis transforms as register FFTs (mixed path): the
    // matrices' factors, forward and inverse; null when they do not apply
    lp::DftFac dfac[2]{};
    const lp::DftFac *dff = nullptr, *dfi = nullptr;
    void *P = nullptr;                                       // R precision
    unsigned *PI = nullptr;
    float *LW = nullptr;            // line-tiled weight table (mixed path)
    // convolution form of the mixed contraction: omega factors C[7][n^3],
    // twiddles and the scratch of fq_bs cells
    float *FQC = nullptr;
    float2 *fscr = nullptr;
    int fq_bs = 0;
    int fq_form = 1;  // 1: fused (axis-2 spectra on chip), 0: three passes through DRAM
    lp::FftTw ftw{};
    // the same form in FP64 for the FP64 path: omega factors, twiddles and
    // the scratch of fq64_bs cells (nullptr: the pair form)
    double *FQC64 = nullptr;
    double2 *fscr64 = nullptr;
    int fq64_bs = 0;
    lp::FftTw64 ftw64{};
    // two-species variant: linear weight table (R precision), window offsets,
    // the linear term's workspace and CCt_linear embedded in a 5x5 matrix
    void *WLin = nullptr;
    long long *win_off = nullptr;
    double2 *qlin = nullptr;
    double *cct_lin5 = nullptr;
    cudaStream_t side = nullptr;    // second stream of the line-tiled contraction
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    long long *line_off = nullptr;
    double *ab = nullptr;
    // state and advection
    double *U = nullptr, *U1 = nullptr, *Ut = nullptr, *rt = nullptr, *pb = nullptr, *potc = nullptr,
           *phix = nullptr, *phiy = nullptr, *fields = nullptr, *mpart = nullptr;
    // mixed-path advection: FP32 stage copies, charge partials per block of
    // 128 records (nullptr when nv^3 is not a multiple of 128), reciprocals
    // of the band diagonal
    float *Ufa = nullptr, *Ufb = nullptr;
    double *apart = nullptr, *rdiag = nullptr;
    // increment form (nv^3 a multiple of 128, Poisson matrix small enough for
    // its dense inverse): FP32 copy of U, running FP32 flux sum, FP32 charge
    // partials of that sum, dense inverse of the Poisson matrix
    float *Uf0 = nullptr, *Sf = nullptr, *ipart = nullptr;
    double *Ainv = nullptr;
    // batched runs (lp_batch): per collided cell nu and dt (nullptr: the
    // scalars), and which parts this context holds
    double *cnu = nullptr, *cdt = nullptr;
    bool owns_state = true, collide_on = true, advect_on = true;
    bool has_state = false;
    // collision workspace (Bcap cells) and schedule: cells per pass (<= Bcap)
    // and warps per block of the line-tiled contraction
    int Bcap = 0, nchunk = 0, Bpass = 0, line_warps = 2;
    void *f = nullptr, *f1 = nullptr, *qn = nullptr, *F = nullptr, *t1 = nullptr, *t2 = nullptr, *Qc = nullptr,
         *Y = nullptr, *Z = nullptr;
    double2 *q[4] = {nullptr, nullptr, nullptr, nullptr};
    double *cpart = nullptr, *lam = nullptr, *dU = nullptr;
    // moment reconciliation (mixed path)
    double *gmom = nullptr, *gm_inv = nullptr, *mtpart = nullptr, *mapart = nullptr, *mlam = nullptr;
    double *incpart = nullptr;  // per-block DG moment partials of the fused projection
    // lazy conservation of the mixed one-species path: the nonzero constraint
    // rows in FP32 (C1[0], C2[1..3], C1[4]) and the multipliers of the four
    // stages, lam4[4][5][Bcap]
    float *cf = nullptr;
    double *lam4 = nullptr;
    // the axis-3 projection pass on the tensor cores (mixed path): its shared
    // GEMM operand and the device error flag of its bounded waits
    float *pj3_tab = nullptr, *pj1_tab = nullptr;
    int *tc_err = nullptr;
    // FP32 mode arrays of the four stages (lazy conservation with the
    // convolution form, whose output is FP32-accurate)
    float2 *qf[4] = {nullptr, nullptr, nullptr, nullptr};
    int nrc = 16;
    // adjoint workspace (FP64 contexts, allocated by the first adjoint call)
    struct Adj {
        bool ready = false;
        double2 *F[4] = {nullptr, nullptr, nullptr, nullptr};  // transforms of the stage node values
        double *r1 = nullptr, *r2 = nullptr;                     // Re FS(q1), Re FS(q2)
        double *lf = nullptr, *lqn = nullptr, *ls = nullptr, *ltp = nullptr;
        double2 *lq = nullptr, *tq = nullptr, *lF = nullptr, *qs = nullptr;
        double *mfH = nullptr, *miH = nullptr;  // conjugate transposes of the DFT matrices
        int *nfirst = nullptr, *ncount = nullptr;
        double *Ainv = nullptr, *lrt = nullptr, *lamF = nullptr, *lphix = nullptr, *lphiy = nullptr, *J = nullptr;
        double *dnu = nullptr;  // per collided cell
        // ComputeQ's VJP: 0 the correlation form (omega factors Cp, per-axis
        // DFT matrices Wf / Wi, scratch cscr), 1 the pair-table gather
        int qvjp_form = 0;
        double *Cp = nullptr;
        double2 *Wf = nullptr, *Wi = nullptr, *cscr = nullptr;
        double *lU = nullptr, *lU1 = nullptr, *lUt = nullptr, *lH = nullptr, *lC = nullptr, *Ukeep = nullptr;
        std::vector<double *> ck;  // checkpoints
        double *seg = nullptr;     // states of one checkpoint segment
        int seg_len = 0;
    } adj;
    // x1 slab of a sharded run (lp_slab_create): own x1 rows are local rows
    // 1..slab_nown, rows 0 and slab_nown + 1 are halo copies of the
    // neighbours' edge rows; i1_off is the global x1 row of local row 0 and
    // slab_gnx1 the global row count (0: not a slab).  The global LDG
    // Poisson factors and their solve buffers (gfields: 14 x global cells).
    int i1_off = 0, slab_gnx1 = 0, slab_nown = 0;
    lp::PoissonTables gpois;
    double *gab = nullptr, *gpb = nullptr, *gpotc = nullptr, *gphix = nullptr, *gphiy = nullptr,
           *gfields = nullptr;
    int *gipiv = nullptr;
    unsigned char *ggate = nullptr;
    // lp_collision_step_host: two staging states used by alternate calls,
    // copy streams, per (staging buffer, chunk) events, and the captured
    // collision of each (staging buffer, cell range)
    cudaStream_t h2d = nullptr, d2h = nullptr;
    double *hstage[2] = {nullptr, nullptr};
    int hnext = 0;
    cudaEvent_t hev_in[2][kHostChunksMax] = {}, hev_col[2][kHostChunksMax] = {}, hev_rest[2] = {},
                hev_free[2] = {};
    struct HostGraph {
        int b, c0, c1;
        cudaGraphExec_t g;
    };
    std::vector<HostGraph> hgraphs;
    // captured step, and captured collision step of all collided cells
    cudaGraphExec_t gexec = nullptr, cgexec = nullptr;
    int cg_kernels = 0;  // kernel nodes of the captured collision step
    int cg_pdl = 0;      // its programmatic kernel-to-kernel edges
    cudaStream_t gstream = nullptr, cgstream = nullptr;
};

namespace {

constexpr int kMomBlocks = 240;

// Programmatic kernel-to-kernel edges in a captured step graph.  Each edge
// from one kernel node to another becomes a programmatic dependency on the
// upstream kernel's `port`: the downstream grid may be launched before the
// upstream kernel has completed (once its blocks have all exited, or all
// started).  Every kernel of the library starts with lp_grid_wait, which holds its
// blocks until the upstream grids have completed and their writes are
// visible, so the graph keeps stream order.  Edges to or from other nodes
// (copies, memsets) stay as captured.
cudaError_t make_edges_programmatic(cudaGraph_t g, int port, int *nconv) {
    *nconv = 0;
    size_t ne = 0;
    cudaError_t e = cudaGraphGetEdges(g, nullptr, nullptr, nullptr, &ne);
    if (e != cudaSuccess || ne == 0) return e;
    std::vector<cudaGraphNode_t> from(ne), to(ne);
    std::vector<cudaGraphEdgeData> ed(ne);
    e = cudaGraphGetEdges(g, from.data(), to.data(), ed.data(), &ne);
    if (e != cudaSuccess) return e;
    std::vector<cudaGraphNode_t> kf, kt;
    std::vector<cudaGraphEdgeData> kold;
    for (size_t i = 0; i < ne; ++i) {
        cudaGraphNodeType tf, tt;
        if (cudaGraphNodeGetType(from[i], &tf) != cudaSuccess || cudaGraphNodeGetType(to[i], &tt) != cudaSuccess)
            return cudaErrorInvalidValue;
        if (tf != cudaGraphNodeTypeKernel || tt != cudaGraphNodeTypeKernel) continue;
        if (ed[i].type != cudaGraphDependencyTypeDefault || ed[i].from_port != cudaGraphKernelNodePortDefault)
            continue;
        kf.push_back(from[i]);
        kt.push_back(to[i]);
        kold.push_back(ed[i]);
    }
    if (kf.empty()) return cudaSuccess;
    cudaGraphEdgeData pd{};
    pd.from_port = (unsigned char)port;
    pd.type = cudaGraphDependencyTypeProgrammatic;
    const std::vector<cudaGraphEdgeData> knew(kf.size(), pd);
    e = cudaGraphRemoveDependencies(g, kf.data(), kt.data(), kold.data(), kf.size());
    if (e != cudaSuccess) return e;
    e = cudaGraphAddDependencies(g, kf.data(), kt.data(), knew.data(), kf.size());
    if (e != cudaSuccess) {
        cudaGraphAddDependencies(g, kf.data(), kt.data(), kold.data(), kf.size());
        return e;
    }
    *nconv = (int)kf.size();
    return cudaSuccess;
}

// Instantiates a captured step graph.  LP_PDL in the environment at capture
// selects programmatic kernel-to-kernel edges: 1 from the upstream kernel's
// programmatic port (the next grid is launched as the last upstream block
// exits), 2 from its launch-completion port (as the last upstream block
// starts); unset or 0 keeps the edges as captured.  On GB300 at 64 cells,
// n = 24, the collision step takes the same time with port 1 and 5% longer
// with port 2 (the next grids' waiting blocks are placed while the current
// kernel runs), so ordinary edges are the default.  A refused edge update or
// instantiation falls back to the graph as captured.  *pdl_edges: the
// programmatic edges of the instantiated graph.
cudaError_t instantiate_step_graph(cudaGraphExec_t *exec, cudaGraph_t g, int *pdl_edges = nullptr) {
    if (pdl_edges) *pdl_edges = 0;
    const char *env = std::getenv("LP_PDL");
    if (env && (env[0] == '1' || env[0] == '2')) {
        const int port = env[0] == '2' ? cudaGraphKernelNodePortLaunchCompletion
                                       : cudaGraphKernelNodePortProgrammatic;
        cudaGraph_t pg = nullptr;
        if (cudaGraphClone(&pg, g) == cudaSuccess) {
            int nconv = 0;
            cudaError_t e = make_edges_programmatic(pg, port, &nconv);
            if (e == cudaSuccess) e = cudaGraphInstantiate(exec, pg, 0);
            cudaGraphDestroy(pg);
            if (e == cudaSuccess) {
                if (pdl_edges) *pdl_edges = nconv;
                return e;
            }
            *exec = nullptr;
        }
        cudaGetLastError();  // a refused update or instantiation leaves no sticky error
    }
    return cudaGraphInstantiate(exec, g, 0);
}

lp_status fail(lp_ctx *c, lp_status s, const std::string &msg) {
    if (c) c->err = msg;
    return s;
}

lp_status cuda_fail(lp_ctx *c, cudaError_t e, const char *where) {
    return fail(c, LP_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define LP_CUDA(call)                                          \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
    } while (0)

template <typename T> lp_status dalloc(lp_ctx *c, T **p, size_t count) {
    void *d = nullptr;
    size_t b = sizeof(T) * (count ? count : 1);
    cudaError_t e = cudaMalloc(&d, b);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(c, LP_ERR_ALLOC, "cudaMalloc of " + std::to_string(b) + " bytes failed");
    }
    c->allocs.push_back(d);
    c->bytes += b;
    *p = static_cast<T *>(d);
    return LP_OK;
}

template <typename T> lp_status upload(lp_ctx *c, T **p, const T *host, size_t count) {
    lp_status s = dalloc(c, p, count);
    if (s != LP_OK) return s;
    LP_CUDA(cudaMemcpy(*p, host, sizeof(T) * count, cudaMemcpyHostToDevice));
    return LP_OK;
}

#define LP_TRY(x)                   \
    do {                            \
        lp_status s_ = (x);         \
        if (s_ != LP_OK) return s_; \
    } while (0)

template <typename R> lp_status upload_real(lp_ctx *c, void **p, const std::vector<double> &v) {
    std::vector<R> h(v.begin(), v.end());
    R *d = nullptr;
    LP_TRY(upload(c, &d, h.data(), h.size()));
    *p = d;
    return LP_OK;
}

inline int round32(int b) { return (b + 31) / 32 * 32; }

template <typename R> lp_status alloc_workspace(lp_ctx *c) {
    using C = typename V2<R>::t;
    const lp::Tables &T = c->T;
    const size_t n3 = T.n3, Bp = c->Bcap, n = T.n, nv = T.nv;
    R *f, *f1, *qn;
    C *F, *t1, *t2, *Qc, *Y, *Z;
    LP_TRY(dalloc(c, &f, n3 * Bp));
    LP_TRY(dalloc(c, &f1, n3 * Bp));
    LP_TRY(dalloc(c, &qn, n3 * Bp));
    LP_TRY(dalloc(c, &F, n3 * Bp));
    LP_TRY(dalloc(c, &t1, n3 * Bp));
    LP_TRY(dalloc(c, &t2, n3 * Bp));
    LP_TRY(dalloc(c, &Qc, n3 * Bp));
    LP_TRY(dalloc(c, &Y, 3 * n * n * nv * Bp));
    LP_TRY(dalloc(c, &Z, 5 * n * nv * nv * Bp));
    c->f = f; c->f1 = f1; c->qn = qn; c->F = F; c->t1 = t1; c->t2 = t2; c->Qc = Qc; c->Y = Y; c->Z = Z;
    for (int i = 0; i < 4; ++i) LP_TRY(dalloc(c, &c->q[i], n3 * Bp));
    c->nchunk = 256;  // point chunks of the FP64 moment sums (parallel partials)
    LP_TRY(dalloc(c, &c->cpart, (size_t)c->nchunk * 5 * Bp));
    LP_TRY(dalloc(c, &c->lam, 5 * Bp));
    LP_TRY(dalloc(c, &c->dU, (size_t)T.nv3 * 5 * Bp));
    if (c->mixed) {
        LP_TRY(upload(c, &c->gmom, T.gmom.data(), T.gmom.size()));
        LP_TRY(upload(c, &c->gm_inv, T.gm_inv, 25));
        LP_TRY(dalloc(c, &c->mtpart, (size_t)c->nchunk * 5 * Bp));
        LP_TRY(dalloc(c, &c->mapart, (size_t)c->nrc * 5 * Bp));
        LP_TRY(dalloc(c, &c->mlam, 5 * Bp));
        LP_TRY(dalloc(c, &c->incpart, (size_t)lp::project_inc_blocks(T.n, T.nv) * 5 * Bp));
        if (lp::fftq_supported(T.n)) {
            std::vector<float> cf(5 * n3);
            for (size_t k = 0; k < n3; ++k) {
                cf[k] = (float)T.c1[k];
                for (int r = 1; r < 4; ++r) cf[r * n3 + k] = (float)T.c2[r * n3 + k];
                cf[4 * n3 + k] = (float)T.c1[4 * n3 + k];
            }
            LP_TRY(upload(c, &c->cf, cf.data(), cf.size()));
            LP_TRY(dalloc(c, &c->lam4, 4 * 5 * Bp));
            for (int i = 0; i < 4; ++i) LP_TRY(dalloc(c, &c->qf[i], n3 * Bp));
        }
    }
    return LP_OK;
}

template <typename R> lp_status upload_tables(lp_ctx *c) {
    const lp::Tables &T = c->T;
    LP_TRY(upload(c, &c->eta, T.eta.data(), T.eta.size()));
    LP_TRY(upload(c, &c->shat, T.shat.data(), T.shat.size()));
    LP_TRY(upload(c, &c->ahat, T.ahat.data(), T.ahat.size()));
    LP_TRY(upload(c, &c->rzero, T.rzero.data(), T.rzero.size()));
    LP_TRY(upload(c, &c->cw, T.cw.data(), T.cw.size()));
    LP_TRY(upload(c, &c->c1, T.c1.data(), T.c1.size()));
    LP_TRY(upload(c, &c->c2, T.c2.data(), T.c2.size()));
    LP_TRY(upload(c, &c->cct, T.cct_inv, 25));
    LP_TRY(upload(c, &c->nodecell, T.nodecell.data(), T.nodecell.size()));
    LP_TRY(upload(c, &c->nodeoff, T.nodeoff.data(), T.nodeoff.size()));
    LP_TRY(upload(c, &c->pair_off, T.pair_off.data(), T.pair_off.size()));
    LP_TRY(upload_real<R>(c, &c->tfac, T.tfac));
    // the axis-3 and axis-1 projection passes on the tensor cores: their
    // shared GEMM operands from the FP32 factors (LP_PJ3_TC=0 in the
    // environment keeps the CUDA-core passes, for comparisons)
    const char *tcenv = std::getenv("LP_PJ3_TC");
    if (c->mixed && !(tcenv && tcenv[0] == '0') && lp::pj3_tc_np(T.nv) <= 256 &&
        (T.n == 8 || T.n == 16 || T.n == 24 || T.n == 32)) {
        std::vector<float> tf(T.tfac.size()), tab;
        for (size_t i = 0; i < tf.size(); ++i) tf[i] = (float)T.tfac[i];
        lp::pj3_tc_table(tf.data(), T.n, T.nv, tab);
        LP_TRY(upload(c, &c->pj3_tab, tab.data(), tab.size()));
        if (T.nv <= 32 && T.nv % 2 == 0) {
            lp::pj1_tc_table(tf.data(), T.n, T.nv, tab);
            LP_TRY(upload(c, &c->pj1_tab, tab.data(), tab.size()));
        }
    }
    if (c->mixed) {  // error flag of the bounded waits (tensor-core projection, fused convolution)
        LP_TRY(dalloc(c, &c->tc_err, 1));
        LP_CUDA(cudaMemset(c->tc_err, 0, sizeof(int)));
    }
    LP_TRY(upload_real<R>(c, &c->mfwd, T.mfwd));
    LP_TRY(upload_real<R>(c, &c->minv, T.minv));
    if (c->mixed && T.dft_fac_ok && (T.n == 8 || T.n == 16 || T.n == 24 || T.n == 32)) {
        for (int d = 0; d < 2; ++d) {
            lp::DftFac &D = c->dfac[d];
            D.n = T.n;
            D.sign = d == 0 ? -1 : 1;
            for (int i = 0; i < T.n; ++i) {
                D.pre[i] = make_float2((float)T.dpre[d][2 * i], (float)T.dpre[d][2 * i + 1]);
                D.post[i] = make_float2((float)T.dpost[d][2 * i], (float)T.dpost[d][2 * i + 1]);
                D.w[i] = make_float2((float)T.dw[d][2 * i], (float)T.dw[d][2 * i + 1]);
            }
        }
        c->dff = &c->dfac[0];
        c->dfi = &c->dfac[1];
    }
    if (c->mixed && lp::lines_supported(T.n)) {
        std::vector<long long> off;
        const long long nw = lp::lines_table_floats(T.n, off);
        LP_TRY(upload(c, &c->line_off, off.data(), off.size()));
        LP_TRY(dalloc(c, &c->LW, (size_t)nw));
        LP_CUDA(lp::launch_lines_table(c->eta, c->shat, c->ahat, c->rzero, c->cw, c->line_off, T.n, c->LW,
                                       c->stream));
        if (lp::fftq_supported(T.n)) {
            std::vector<float> C;
            lp::fftq_coefficients(T.shat.data(), T.ahat.data(), T.cw.data(), T.h_eta, T.n, C);
            LP_TRY(upload(c, &c->FQC, C.data(), C.size()));
            // chunk of cells of one convolution pass: 64, or more while the
            // scratch stays within 512 MB
            const size_t per_cell = lp::fftq_scratch_elems(T.n, 1) * sizeof(float2);
            const int fit = (int)std::min<size_t>((size_t)c->Bcap, (512ull << 20) / per_cell) / 32 * 32;
            c->fq_bs = std::min(c->Bcap, std::max(64, fit));
            // LP_FQ_CHUNK=<cells> (a multiple of 32) in the environment sets a
            // smaller chunk: the intermediates of a smaller chunk stay in L2
            // between the convolution's kernels
            if (const char *cenv = std::getenv("LP_FQ_CHUNK")) {
                const int v = std::atoi(cenv) / 32 * 32;
                if (v >= 32 && v < c->fq_bs) c->fq_bs = v;
            }
            LP_TRY(dalloc(c, &c->fscr, lp::fftq_scratch_elems(T.n, c->fq_bs)));
            c->ftw = lp::fftq_twiddles(T.n);
            // the fused convolution (LP_FQ_FUSED=0 in the environment keeps
            // the three passes through DRAM, for comparisons)
            const char *fenv = std::getenv("LP_FQ_FUSED");
            c->fq_form = (fenv && fenv[0] == '0') ? 0 : 1;
            // the convolution form is the faster one from n = 16 up
            if (T.n >= 16) c->line_warps = 0;
        }
    } else {
        const size_t npair = (size_t)T.pair_off[T.n3];
        R *P = nullptr;
        LP_TRY(dalloc(c, &P, npair));
        LP_TRY(dalloc(c, &c->PI, npair));
        c->P = P;
        LP_CUDA(lp::launch_pairs(c->eta, c->shat, c->ahat, c->rzero, c->cw, c->pair_off, T.n,
                                 std::is_same<R, double>::value ? (double *)P : nullptr,
                                 std::is_same<R, float>::value ? (float *)P : nullptr, c->PI, c->stream));
        // FP64 path: the convolution form in FP64 where the node grid is
        // uniform.  The form needs eta(xi) - eta(omega) = (xi - omega) h_eta;
        // with defect F11 left in (n = 24) the middle node is 8.9e-16 instead
        // of 0, the weight there is that of a node off zero, and the pair form
        // (the reference's own evaluation) is kept.  Elsewhere the two forms
        // agree to 1e-14 (relative L2) at every n.  LP_FQ64=0 in the
        // environment keeps the pair form, for comparisons.
        const char *fenv = std::getenv("LP_FQ64");
        if (!c->mixed && lp::fftq_supported(T.n) && T.eta[T.n / 2] == 0.0 && !(fenv && fenv[0] == '0')) {
            std::vector<double> C;
            lp::fftq_coefficients64(T.shat.data(), T.ahat.data(), T.cw.data(), T.h_eta, T.n, C);
            LP_TRY(upload(c, &c->FQC64, C.data(), C.size()));
            // chunks of 32 cells or more while the scratch stays within 512 MB
            const size_t per_cell = lp::fftq_scratch_elems64(T.n, 1) * sizeof(double2);
            const int fit = (int)std::min<size_t>((size_t)c->Bcap, (512ull << 20) / per_cell) / 32 * 32;
            c->fq64_bs = std::min(c->Bcap, std::max(32, fit));
            LP_TRY(dalloc(c, &c->fscr64, lp::fftq_scratch_elems64(T.n, c->fq64_bs)));
            c->ftw64 = lp::fftq_twiddles64(T.n);
        }
    }
    if (T.prm.linear_ei) {
        LP_TRY(upload(c, &c->win_off, T.win_off.data(), T.win_off.size()));
        LP_TRY(upload(c, &c->cct_lin5, T.cct_lin5, 25));
        const size_t nw = (size_t)T.win_off[T.n3];
        R *W = nullptr;
        LP_TRY(dalloc(c, &W, nw));
        c->WLin = W;
        LP_CUDA(lp::launch_lin_weights(c->eta, c->shat, c->cw, c->win_off, T.n, T.scale3,
                                       std::is_same<R, double>::value ? (double *)W : nullptr,
                                       std::is_same<R, float>::value ? (float *)W : nullptr, c->stream));
        LP_TRY(dalloc(c, &c->qlin, (size_t)T.n3 * c->Bcap));
    }
    return alloc_workspace<R>(c);
}

// Poisson tables and the advection buffers; U, U1, Ut are allocated unless
// the context works on a batch's state buffers (owns_state false).
lp_status setup_advection(lp_ctx *c) {
    const lp::Tables &T = c->T;
    const size_t rec = (size_t)T.size * 7, nc = T.ncell;
    LP_TRY(upload(c, &c->ab, T.pois.ab.data(), T.pois.ab.size()));
    LP_TRY(upload(c, &c->ipiv, T.pois.ipiv.data(), T.pois.ipiv.size()));
    LP_TRY(upload(c, &c->gate, T.pois.gate.data(), T.pois.gate.size()));
    LP_TRY(dalloc(c, &c->rt, 3 * nc));
    LP_TRY(dalloc(c, &c->pb, (size_t)T.pois.ndim));
    LP_TRY(dalloc(c, &c->potc, 3 * nc));
    LP_TRY(dalloc(c, &c->phix, 3 * nc));
    LP_TRY(dalloc(c, &c->phiy, 3 * nc));
    LP_TRY(dalloc(c, &c->fields, 14 * nc));
    if (c->mixed) {
        LP_TRY(dalloc(c, &c->Ufa, rec));
        LP_TRY(dalloc(c, &c->Ufb, rec));
        if (T.nv3 % 128 == 0) LP_TRY(dalloc(c, &c->apart, 3 * ((size_t)T.size / 128)));
        // reciprocals of the diagonal of the band factor U (row ku+kl+1 of AB)
        const lp::PoissonTables &pt = T.pois;
        std::vector<double> rd(pt.ndim);
        for (int j = 0; j < pt.ndim; ++j) rd[j] = 1.0 / pt.ab[(size_t)(pt.kl + pt.ku) + (size_t)j * pt.ldab];
        LP_TRY(upload(c, &c->rdiag, rd.data(), rd.size()));
        if (c->apart && pt.ndim <= 4096) {
            LP_TRY(dalloc(c, &c->Uf0, rec));
            LP_TRY(dalloc(c, &c->Sf, rec));
            LP_TRY(dalloc(c, &c->ipart, 3 * ((size_t)T.size / 128)));
            std::vector<double> inv;
            lp::poisson_inverse(pt, inv);
            LP_TRY(upload(c, &c->Ainv, inv.data(), inv.size()));
        }
    }
    return LP_OK;
}

lp::PoissonDev poisson_dev_of(const lp::PoissonTables &p, const double *ab, const int *ipiv,
                              const unsigned char *gate) {
    lp::PoissonDev d{};
    d.nx = p.nx; d.ny = p.ny; d.ndim = p.ndim; d.kl = p.kl; d.ku = p.ku; d.ldab = p.ldab;
    d.ab = ab; d.ipiv = ipiv; d.dxp = p.dxp; d.dyp = p.dyp; d.gate = gate;
    std::memcpy(d.blk[0], p.acvx, sizeof(p.acvx));
    std::memcpy(d.blk[1], p.acyrr, sizeof(p.acyrr));
    std::memcpy(d.blk[2], p.acyrl, sizeof(p.acyrl));
    std::memcpy(d.blk[3], p.acvy, sizeof(p.acvy));
    std::memcpy(d.blk[4], p.acxrr, sizeof(p.acxrr));
    std::memcpy(d.blk[5], p.acxrl, sizeof(p.acxrl));
    d.rdiag = nullptr;
    d.rdxp = 1.0 / p.dxp; d.rdyp = 1.0 / p.dyp;
    d.cscale = 1.0;
    return d;
}

// fast = false: the host's operations (pois2d bit for bit); fast = true: the
// mixed path's variant (reciprocals, charge from block partials).
lp::PoissonDev poisson_dev(const lp_ctx *c, bool fast) {
    lp::PoissonDev d = poisson_dev_of(c->T.pois, c->ab, c->ipiv, c->gate);
    d.rdiag = fast ? c->rdiag : nullptr;
    d.cscale = (fast && c->apart) ? c->T.scalev : 1.0;
    return d;
}

lp::AdvectDev advect_dev(const lp_ctx *c) {
    const lp::Tables &T = c->T;
    lp::AdvectDev a{};
    a.nx1 = T.prm.nx1; a.nx2 = T.prm.nx2; a.nv = T.nv; a.size = T.size;
    a.lv = T.prm.lv; a.dv = T.dv; a.dx = T.dx; a.scalev = T.scalev; a.dt = T.prm.dt;
    a.rdv = 1.0 / T.dv; a.inv = 1.0 / T.dx / T.scalev;
    a.dt_f = (float)T.prm.dt; a.dt6 = T.prm.dt / 6.;
    a.f.lv = (float)a.lv; a.f.dv = (float)a.dv; a.f.rdv = (float)a.rdv; a.f.scalev = (float)a.scalev;
    a.f.inv = (float)a.inv;
    a.fscale = (T.prm.fixes & LP_FIX_F12) ? T.dx : 1.0;
    a.f.fscale = (float)a.fscale;
    return a;
}

// pois2d on stage values Us with the host's operations (the FP64 path and
// the reference-shaped lp_poisson).
lp_status poisson_on(lp_ctx *c, const double *Us) {
    LP_CUDA(lp::launch_charge(Us, c->T.ncell, c->T.nv3, c->T.scalev, c->rt, c->stream));
    LP_CUDA(lp::launch_poisson(poisson_dev(c, false), c->rt, 1, c->pb, c->potc, c->phix, c->phiy, c->fields,
                               c->stream));
    return LP_OK;
}

// Mixed path: Poisson solve whose charge is in c->apart (block partials of
// the stage values, written by the previous kernel) or, when the records of
// a block can straddle cells, summed from Us here.
lp_status poisson_mixed(lp_ctx *c, const double *Us) {
    const int npart = c->apart ? c->T.nv3 / 128 : 1;
    if (!c->apart) LP_CUDA(lp::launch_charge(Us, c->T.ncell, c->T.nv3, c->T.scalev, c->rt, c->stream));
    LP_CUDA(lp::launch_poisson(poisson_dev(c, true), c->apart ? c->apart : c->rt, npart, c->pb, c->potc, c->phix,
                               c->phiy, c->fields, c->stream));
    return LP_OK;
}

// One SSP-RK3 step of U (RK3, A:428-601): stage buffers U -> U1 -> Ut -> U.
// FP64 path: every flux in FP64, each Poisson solve as the reference's.
// Mixed path: fluxes in FP32 from FP32 stage copies, the stage combinations,
// charge sums and Poisson solves in FP64.
lp_status advect(lp_ctx *c) {
    NvtxRange r("RK3 advection + LDG Poisson");
    const lp::AdvectDev ad = advect_dev(c);
    if (!c->mixed) {
        LP_TRY(poisson_on(c, c->U));
        LP_CUDA(lp::launch_flux_stage(ad, c->U, c->U, nullptr, c->fields, 0, c->U1, nullptr, nullptr, c->stream));
        LP_TRY(poisson_on(c, c->U1));
        LP_CUDA(lp::launch_flux_stage(ad, c->U, c->U1, nullptr, c->fields, 1, c->Ut, nullptr, nullptr, c->stream));
        LP_TRY(poisson_on(c, c->Ut));
        LP_CUDA(lp::launch_flux_stage(ad, c->U, c->Ut, nullptr, c->fields, 2, c->U, nullptr, nullptr, c->stream));
        return LP_OK;
    }
    if (c->Ainv) {
        // increment form: U1 = U + dt H0, U2 = U + dt/4 (H0 + H1), U += dt/6 (H0 + H1 + 4 H2)
        const lp::PoissonDev pd = poisson_dev(c, true);
        const int npart = c->T.nv3 / 128;
        const double dt = c->T.prm.dt;
        LP_CUDA(lp::launch_state_f32_grp(c->U, c->T.size, c->Uf0, c->apart, c->stream));
        LP_CUDA(lp::launch_poisson_dense(pd, c->apart, nullptr, 0., npart, c->Ainv, c->pb, c->potc, c->phix,
                                         c->phiy, c->fields, c->stream));
        LP_CUDA(lp::launch_flux_inc(ad, 0, c->Uf0, c->Uf0, c->fields, c->Sf, c->Ufa, c->U, c->ipart, c->stream));
        LP_CUDA(lp::launch_poisson_dense(pd, c->apart, c->ipart, dt, npart, c->Ainv, c->pb, c->potc, c->phix,
                                         c->phiy, c->fields, c->stream));
        LP_CUDA(lp::launch_flux_inc(ad, 1, c->Ufa, c->Uf0, c->fields, c->Sf, c->Ufb, c->U, c->ipart, c->stream));
        LP_CUDA(lp::launch_poisson_dense(pd, c->apart, c->ipart, 0.25 * dt, npart, c->Ainv, c->pb, c->potc,
                                         c->phix, c->phiy, c->fields, c->stream));
        LP_CUDA(lp::launch_flux_inc(ad, 2, c->Ufb, c->Uf0, c->fields, c->Sf, nullptr, c->U, nullptr, c->stream));
        return LP_OK;
    }
    LP_CUDA(lp::launch_state_f32(c->U, c->T.size, c->Ufa, c->apart, c->stream));
    LP_TRY(poisson_mixed(c, c->U));
    LP_CUDA(lp::launch_flux_stage(ad, c->U, c->U, c->Ufa, c->fields, 0, c->U1, c->Ufb, c->apart, c->stream));
    LP_TRY(poisson_mixed(c, c->U1));
    LP_CUDA(lp::launch_flux_stage(ad, c->U, c->U1, c->Ufb, c->fields, 1, c->Ut, c->Ufa, c->apart, c->stream));
    LP_TRY(poisson_mixed(c, c->Ut));
    LP_CUDA(lp::launch_flux_stage(ad, c->U, c->Ut, c->Ufa, c->fields, 2, c->U, nullptr, nullptr, c->stream));
    return LP_OK;
}

// The weighted contraction of ComputeQ on the transformed node values F.
// Mixed path: line_warps 0 selects the convolution form, 2 or 4 the
// line-tiled weighted sum with that many warps per line.
// q32: the convolution form writes the mode array in FP32 there.
// lam (with q32): conserveAllMoments' multipliers of the FP32 mode array,
// [5][Bp], from the constraint sums of the convolution form's last kernel.
template <typename R> lp_status contract(lp_ctx *c, int Bp, double2 *q, float2 *q32 = nullptr,
                                         double *lam = nullptr) {
    using C = typename V2<R>::t;
    const lp::Tables &T = c->T;
    if constexpr (std::is_same<R, double>::value) {
        if (c->FQC64 && !q32) {
            for (int c0 = 0; c0 < Bp; c0 += c->fq64_bs)
                LP_CUDA(lp::launch_computeq_fft64((const double2 *)c->F, c->FQC64, c->ftw64, T.n, Bp, c0,
                                                  std::min(c->fq64_bs, Bp - c0), c->fscr64, c->fq64_bs, q,
                                                  c->stream));
            return LP_OK;
        }
    }
    if (c->FQC && c->line_warps == 0) {
        lp::ConsFused cons;
        if (lam) {
            if (!q32 || !c->cf || lp::fftq_cons_blocks(T.n) > c->nchunk)
                return fail(c, LP_ERR_INVALID, "fused conservation sums need FP32 mode arrays");
            cons.cf = c->cf;
            cons.part = c->cpart;
        }
        for (int c0 = 0; c0 < Bp; c0 += c->fq_bs)
            LP_CUDA(lp::launch_computeq_fft((const float2 *)c->F, c->FQC, c->ftw, T.n, Bp, c0,
                                            std::min(c->fq_bs, Bp - c0), c->fscr, c->fq_bs, q, c->stream, -1,
                                            q32, lam ? &cons : nullptr, c->fq_form, c->tc_err));
        if (lam) LP_CUDA(lp::launch_cons_lambda(c->cpart, lp::fftq_cons_blocks(T.n), c->cct, Bp, lam, c->stream));
        return LP_OK;
    }
    if (q32) return fail(c, LP_ERR_INVALID, "FP32 mode arrays need the convolution form");
    if (c->LW) {
        // the k-tiles run on two streams so that the short lines at the end
        // of one tile overlap the next tile
        if (c->side) {
            LP_CUDA(cudaEventRecord(c->ev_fork, c->stream));
            LP_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
        }
        LP_CUDA(lp::launch_computeq_lines((const float2 *)c->F, c->LW, c->line_off, T.n, Bp, q, c->stream,
                                          c->line_warps, c->side));
        if (c->side) {
            LP_CUDA(cudaEventRecord(c->ev_join, c->side));
            LP_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
        }
        return LP_OK;
    }
    LP_CUDA(lp::launch_computeq<R>((const C *)c->F, (const R *)c->P, c->PI, c->pair_off, T.n3, Bp, q, c->stream));
    return LP_OK;
}

// The conserved mode array of one stage from the transformed node values F:
// ComputeQ's contraction and conserveAllMoments; in the two-species variant
// the linear term is added before, conserved with its own two constraints,
// and added again after (C:551-635, K:63-98, C:656-698).
// slot >= 0 (lazy conservation): only the multipliers of stage `slot` are
// computed, into lam4; the consumers of q apply the correction on load.
// q32 (with slot): the mode array is kept in FP32 there.
template <typename R> lp_status stage_q(lp_ctx *c, int Bp, double2 *q, int slot = -1, float2 *q32 = nullptr) {
    using C = typename V2<R>::t;
    const lp::Tables &T = c->T;
    if (q32) return contract<R>(c, Bp, q, q32, c->lam4 + slot * 5 * Bp);
    LP_TRY(contract<R>(c, Bp, q, q32));
    if (c->WLin) {
        const long long tot = (long long)T.n3 * Bp;
        LP_CUDA(lp::launch_qlin<R>((const C *)c->F, (const R *)c->WLin, c->win_off, T.n, Bp, c->qlin, c->stream));
        LP_CUDA(lp::launch_qadd(q, c->qlin, tot, c->stream));
        LP_CUDA(lp::launch_conserve(q, c->c1, c->c2, c->cct, T.n3, Bp, c->cpart, c->nchunk, c->lam, c->stream));
        LP_CUDA(lp::launch_conserve(c->qlin, c->c1, c->c2, c->cct_lin5, T.n3, Bp, c->cpart, c->nchunk, c->lam,
                                    c->stream));
        LP_CUDA(lp::launch_qadd(q, c->qlin, tot, c->stream));
        return LP_OK;
    }
    if (slot >= 0) {
        LP_CUDA(lp::launch_conserve(q, c->c1, c->c2, c->cct, T.n3, Bp, c->cpart, c->nchunk, c->lam4 + slot * 5 * Bp,
                                    c->stream, false));
        return LP_OK;
    }
    LP_CUDA(lp::launch_conserve(q, c->c1, c->c2, c->cct, T.n3, Bp, c->cpart, c->nchunk, c->lam, c->stream));
    return LP_OK;
}

// RK4 stages 1-3 (C:831-865) from node values f and conserved q[0].
lp::Rates rates_at(const lp_ctx *c, int c0) {
    lp::Rates r;
    if (c->cnu) { r.nu = c->cnu + c0; r.dt = c->cdt + c0; }
    return r;
}

// lazy: the stages' conservation corrections are applied by the consumers
// (the next FS pass and the first DG projection pass).
// f32 (with lazy): the mode arrays are the FP32 ones, c->qf.
template <typename R> lp_status rk4_stages(lp_ctx *c, int c0, int Bp, bool lazy = false, bool f32 = false) {
    using C = typename V2<R>::t;
    const lp::Tables &T = c->T;
    const R *M = (const R *)c->mfwd, *Mi = (const R *)c->minv;
    for (int s = 0; s < 3; ++s) {
        if (f32) {
            LP_CUDA(lp::launch_fs_fwd32(c->qf[s], (float2 *)c->t1, (float2 *)c->t2, (float2 *)c->F,
                                        (const float *)Mi, (const float *)M, T.n, Bp, s, T.prm.dt, T.prm.nu,
                                        (const float *)c->f, (float *)c->qn, (float *)c->f1, c->stream,
                                        rates_at(c, c0), c->cf, c->lam4 + s * 5 * Bp, c->dfi, c->dff));
        } else {
            LP_CUDA(lp::launch_fs_stage<R>(c->q[s], (C *)c->t1, (C *)c->t2, Mi, T.n, Bp, s, T.prm.dt, T.prm.nu,
                                           (const R *)c->f, (R *)c->qn, (R *)c->f1, c->stream, rates_at(c, c0),
                                           lazy ? c->cf : nullptr, lazy ? c->lam4 + s * 5 * Bp : nullptr, c->dfi));
            LP_CUDA(lp::launch_fwd<R>((const R *)c->f1, (C *)c->t1, (C *)c->F, M, T.n, Bp, c->stream, c->dff));
        }
        LP_TRY(stage_q<R>(c, Bp, c->q[s + 1], lazy ? s + 1 : -1, f32 ? c->qf[s + 1] : nullptr));
    }
    return LP_OK;
}

// defer_fix: the mixed path's moment correction is left to the scatter.
// The DG moments of the increment are linear functionals of the RK4
// combination of q0..q3; every q_s leaves conserveAllMoments with zero mass,
// momentum and energy integrals, and the DG projection keeps those integrals
// (1, v and |v|^2 lie in the span of each cell's basis), so the FP64 target
// of the one-species operator is zero and the correction only removes the
// FP32 projection's moment error.  The two-species operator conserves only
// mass and energy of its linear term: its target is summed from q0..q3.
template <typename R> lp_status project(lp_ctx *c, int c0, int B, int Bp, bool defer_fix = false) {
    using C = typename V2<R>::t;
    const lp::Tables &T = c->T;
    static const int fixed_slots[5] = {0, 3, 4, 5, 6}, ref_slots[5] = {0, 2, 3, 4, 5};
    const bool f1 = (T.prm.fixes & LP_FIX_F1) != 0;
    const bool fix = c->mixed && f1;
    const bool target = fix && c->WLin;
    // the FP64 target moments need only q0..q3: on the side stream, beside the projection
    cudaStream_t tst = (target && c->side) ? c->side : c->stream;
    if (target) {
        if (tst != c->stream) {
            LP_CUDA(cudaEventRecord(c->ev_fork, c->stream));
            LP_CUDA(cudaStreamWaitEvent(tst, c->ev_fork, 0));
        }
        LP_CUDA(lp::launch_moment_target(c->q[0], c->q[1], c->q[2], c->q[3], T.prm.nu, c->gmom, T.n3, Bp, c->nchunk,
                                         c->mtpart, tst, rates_at(c, c0)));
        if (tst != c->stream) LP_CUDA(cudaEventRecord(c->ev_join, tst));
    }
    LP_CUDA(lp::launch_project<R>(c->q[0], c->q[1], c->q[2], c->q[3], T.prm.nu, (const R *)c->tfac, T.n, T.nv, Bp,
                                  B, c0, c->U, f1 ? 7 : 6, f1 ? fixed_slots : ref_slots, T.prm.dt, T.scalev,
                                  T.scaleL, T.scale3, (C *)c->Qc, (C *)c->Y, (C *)c->Z, c->dU, c->stream,
                                  rates_at(c, c0)));
    if (fix) {
        if (tst != c->stream) LP_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
        const double kfac = 1. / T.scalev / T.scaleL / T.scale3;
        LP_CUDA(lp::launch_moment_finish(target ? c->mtpart : nullptr, c->nchunk, c->U, T.nv, T.dv, T.prm.lv, c0, B,
                                         Bp, c->nrc, c->mapart, c->gm_inv, T.prm.dt * kfac, kfac, c->mlam, c->dU,
                                         c->stream, rates_at(c, c0), !defer_fix));
    }
    return LP_OK;
}

// The mixed path with LP_FIX_F1 fixed: the DG projection writes the
// coefficient increments and the partial sums of their moments, and the
// multipliers of the moment correction follow; the scatter adds both to U.
bool fused_tail(const lp_ctx *c) { return c->mixed && (c->T.prm.fixes & LP_FIX_F1); }

// Lazy conservation: the one-species mixed path with the fused tail and the
// register-pencil kernels (the two-species operator keeps its add-conserve-add order).
bool lazy_cons(const lp_ctx *c) { return fused_tail(c) && !c->WLin && c->cf; }

lp_status project_fused(lp_ctx *c, int c0, int B, int Bp, bool lazy = false, bool f32 = false) {
    const lp::Tables &T = c->T;
    const bool target = c->WLin != nullptr;
    cudaStream_t tst = (target && c->side) ? c->side : c->stream;
    if (target) {
        if (tst != c->stream) {
            LP_CUDA(cudaEventRecord(c->ev_fork, c->stream));
            LP_CUDA(cudaStreamWaitEvent(tst, c->ev_fork, 0));
        }
        LP_CUDA(lp::launch_moment_target(c->q[0], c->q[1], c->q[2], c->q[3], T.prm.nu, c->gmom, T.n3, Bp, c->nchunk,
                                         c->mtpart, tst, rates_at(c, c0)));
        if (tst != c->stream) LP_CUDA(cudaEventRecord(c->ev_join, tst));
    }
    LP_CUDA(lp::launch_project_inc(c->q[0], c->q[1], c->q[2], c->q[3], T.prm.nu, (const float *)c->tfac, T.n, T.nv,
                                   Bp, B, T.prm.dt, T.scalev, T.scaleL, T.scale3, (float2 *)c->Qc, (float2 *)c->Y,
                                   (float2 *)c->Z, (float *)c->dU, c->incpart, T.prm.lv, T.dv, c->stream, rates_at(c, c0),
                                   lazy ? c->cf : nullptr, lazy ? c->lam4 : nullptr, f32 ? c->qf : nullptr,
                                   c->pj3_tab, c->tc_err, c->pj1_tab));
    if (tst != c->stream) LP_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    const double kfac = 1. / T.scalev / T.scaleL / T.scale3;
    LP_CUDA(lp::launch_lambda_inc(target ? c->mtpart : nullptr, c->nchunk, c->incpart, T.n, T.nv, B, Bp, c->gm_inv,
                                  T.prm.dt * kfac, kfac, c->mlam, c->stream, rates_at(c, c0)));
    return LP_OK;
}

// Collision step of cells [c0, c0+B), B <= Bcap (LP_ompi_1.cpp:502-532).
template <typename R> lp_status collide_batch(lp_ctx *c, int c0, int B) {
    using C = typename V2<R>::t;
    const lp::Tables &T = c->T;
    const int Bp = round32(B);
    const int slot1 = (T.prm.fixes & LP_FIX_F2) ? 3 : 2;
    {
        NvtxRange rn("setInit_spectral + fft3D");
        LP_CUDA(lp::launch_nodes<R>(c->U, T.nv, T.n, c0, B, Bp, slot1, c->nodecell, c->nodeoff, T.dv, (R *)c->f,
                                    c->stream));
        LP_CUDA(lp::launch_fwd<R>((const R *)c->f, (C *)c->t1, (C *)c->F, (const R *)c->mfwd, T.n, Bp, c->stream,
                                  c->dff));
    }
    const bool lazy = lazy_cons(c);
    // FP32 mode arrays: the convolution form's output is FP32-accurate
    const bool f32 = lazy && c->FQC && c->line_warps == 0 && c->qf[0];
    {
        NvtxRange r("ComputeQ + conserveAllMoments, stage 0");
        LP_TRY(stage_q<R>(c, Bp, c->q[0], lazy ? 0 : -1, f32 ? c->qf[0] : nullptr));
    }
    {
        NvtxRange r("RK4 stages 1-3 (FS, fft3D, ComputeQ, conserveAllMoments)");
        LP_TRY(rk4_stages<R>(c, c0, Bp, lazy, f32));
    }
    NvtxRange r("DG projection (IntModes) and moment correction");
    if (fused_tail(c)) return project_fused(c, c0, B, Bp, lazy, f32);
    LP_TRY(project<R>(c, c0, B, Bp, true));
    return LP_OK;
}

// Nodes, forward transform and conserved q[0..3] of cells [c0, c0+B): the
// inputs of every stage, for lp_time_kernel.
template <typename R> lp_status collide_batch_prefix(lp_ctx *c, int c0, int B) {
    using C = typename V2<R>::t;
    const lp::Tables &T = c->T;
    const int Bp = round32(B);
    const int slot1 = (T.prm.fixes & LP_FIX_F2) ? 3 : 2;
    LP_CUDA(lp::launch_nodes<R>(c->U, T.nv, T.n, c0, B, Bp, slot1, c->nodecell, c->nodeoff, T.dv, (R *)c->f,
                                c->stream));
    LP_CUDA(lp::launch_fwd<R>((const R *)c->f, (C *)c->t1, (C *)c->F, (const R *)c->mfwd, T.n, Bp, c->stream,
                              c->dff));
    LP_TRY(stage_q<R>(c, Bp, c->q[0]));
    LP_TRY(rk4_stages<R>(c, c0, Bp));
    return LP_OK;
}

lp_status collide(lp_ctx *c, int c0, int c1) {
    NvtxRange r("collision step");
    // All batches read the pre-collision state (the reference scatters after
    // the loop), so dU of every batch is kept and scattered at the end when
    // the whole range fits one batch; larger ranges are processed batch by
    // batch with the stride-7 read of LP_FIX_F1, which only touches the
    // batch's own records.
    const int total = c1 - c0, pass = c->Bpass;
    for (int b0 = c0; b0 < c1; b0 += pass) {
        const int B = std::min(pass, c1 - b0);
        if (total > pass && !(c->T.prm.fixes & LP_FIX_F1))
            return fail(c, LP_ERR_INVALID, "reference slot reads (F1 unfixed) need all cells in one batch");
        LP_TRY(c->mixed ? collide_batch<float>(c, b0, B) : collide_batch<double>(c, b0, B));
        if (fused_tail(c))
            LP_CUDA(lp::launch_scatter_inc((const float *)c->dU, round32(B), B, c->T.nv, b0, c->U, c->mlam, c->T.dv, c->T.prm.lv,
                                           c->stream));
        else
            LP_CUDA(lp::launch_scatter(c->dU, c->T.nv3, b0, B, c->U, c->stream, nullptr, c->T.nv, c->T.dv,
                                       c->T.prm.lv));
    }
    return LP_OK;
}

lp_status one_step(lp_ctx *c) {
    LP_TRY(advect(c));
    if (c->T.prm.nu > 0.) LP_TRY(collide(c, 0, c->T.ncollide));
    return LP_OK;
}

// Copy a contiguous host vector into column 0 of a cell-minor n3 x 32 buffer.
lp_status put_column(lp_ctx *c, void *dst, size_t elem, const void *src, size_t count) {
    LP_CUDA(cudaMemsetAsync(dst, 0, elem * count * 32, c->stream));
    LP_CUDA(cudaMemcpy2DAsync(dst, elem * 32, src, elem, elem, count, cudaMemcpyHostToDevice, c->stream));
    return LP_OK;
}
lp_status get_column(lp_ctx *c, void *dst, size_t elem, const void *src, size_t pitch, size_t count) {
    LP_CUDA(cudaMemcpy2DAsync(dst, elem, src, pitch, elem, count, cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}

template <typename R> lp_status put_real_column(lp_ctx *c, R *dst, const double *src, size_t count) {
    std::vector<R> h(src, src + count);
    LP_TRY(put_column(c, dst, sizeof(R), h.data(), count));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}
template <typename R> lp_status put_cplx_column(lp_ctx *c, typename V2<R>::t *dst, const double *src, size_t count) {
    std::vector<R> h(src, src + 2 * count);
    LP_TRY(put_column(c, dst, 2 * sizeof(R), h.data(), count));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}
template <typename R> lp_status get_cplx_column(lp_ctx *c, double *dst, const typename V2<R>::t *src, size_t count) {
    std::vector<R> h(2 * count);
    LP_TRY(get_column(c, h.data(), 2 * sizeof(R), src, 32 * 2 * sizeof(R), count));
    for (size_t i = 0; i < 2 * count; ++i) dst[i] = (double)h[i];
    return LP_OK;
}

template <typename R> lp_status do_fft3d(lp_ctx *c, const double *in, double *out, bool inverse) {
    using C = typename V2<R>::t;
    const lp::Tables &T = c->T;
    if (!inverse) {
        LP_TRY(put_cplx_column<R>(c, (C *)c->t2, in, T.n3));
        LP_CUDA(lp::launch_fwd_complex<R>((const C *)c->t2, (C *)c->t1, (C *)c->F, (const R *)c->mfwd, T.n, 32, c->stream));
        return get_cplx_column<R>(c, out, (const C *)c->F, T.n3);
    }
    LP_TRY(put_cplx_column<double>(c, c->q[0], in, T.n3));
    LP_CUDA(lp::launch_fs_full<R>(c->q[0], (C *)c->t1, (C *)c->t2, (C *)c->F, (const R *)c->minv, T.n, 32, c->stream));
    return get_cplx_column<R>(c, out, (const C *)c->F, T.n3);
}

// ComputeQ of one cell; in the two-species variant qhat is Q(f,f) plus the
// linear term and qhat_lin (optional) the linear term alone.
template <typename R> lp_status do_compute_q(lp_ctx *c, const double *f, double *qhat, double *qhat_lin = nullptr) {
    using C = typename V2<R>::t;
    const lp::Tables &T = c->T;
    LP_TRY(put_real_column<R>(c, (R *)c->f, f, T.n3));
    LP_CUDA(lp::launch_fwd<R>((const R *)c->f, (C *)c->t1, (C *)c->F, (const R *)c->mfwd, T.n, 32, c->stream));
    LP_TRY(contract<R>(c, 32, c->q[0]));
    if (c->WLin) {
        LP_CUDA(lp::launch_qlin<R>((const C *)c->F, (const R *)c->WLin, c->win_off, T.n, 32, c->qlin, c->stream));
        LP_CUDA(lp::launch_qadd(c->q[0], c->qlin, (long long)T.n3 * 32, c->stream));
        if (qhat_lin) LP_TRY(get_cplx_column<double>(c, qhat_lin, c->qlin, T.n3));
    }
    return get_cplx_column<double>(c, qhat, c->q[0], T.n3);
}

template <typename R> lp_status do_rk4_cell(lp_ctx *c, const double *f, int cell, const double *qhat, double *dU) {
    const lp::Tables &T = c->T;
    LP_TRY(put_real_column<R>(c, (R *)c->f, f, T.n3));
    LP_TRY(put_cplx_column<double>(c, c->q[0], qhat, T.n3));
    LP_TRY(rk4_stages<R>(c, cell, 32));
    LP_TRY(project<R>(c, cell, 1, 32));
    LP_CUDA(cudaMemcpyAsync(dU, c->dU, sizeof(double) * 5 * T.nv3, cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}

// SetInit_LD (source/SetInit_1.cpp:60-115) and its two variants, on the host.
// i1_off: global x1 index of the context's row 0 (a slab's halo row).
void set_init_host(const lp::Tables &T, int kind, double u, std::vector<double> &U, int i1_off = 0) {
    static const double GW[5] = {0.5688888888888889, 0.4786286704993665, 0.4786286704993665, 0.2369268850561891,
                                 0.2369268850561891};
    static const double GX[5] = {0., -0.5384693101056831, 0.5384693101056831, -0.9061798459386640,
                                 0.9061798459386640};
    const int nv = T.nv, nx1 = T.prm.nx1, nx2 = T.prm.nx2;
    const double a = T.prm.a_amp, cw = T.prm.k_wave, dv = T.dv, dx = T.dx, PI = T.PI, lv = T.prm.lv;
    auto gridv = [&](double m) { return (-lv + (m + 0.5) * dv); };
    auto gridx = [&](double m) { return (m + 0.5) * dx; };
    auto maxw = [&](double v1, double v2, double v3, double Tt) {
        double r2 = v1 * v1 + v2 * v2 + v3 * v3;
        return std::exp(-r2 / (2 * Tt)) / (2 * PI * Tt * std::sqrt(2 * Tt * PI));
    };
    U.assign((size_t)T.size * 7, 0.);
    for (int j1 = 0; j1 < nv; ++j1)
        for (int j2 = 0; j2 < nv; ++j2)
            for (int j3 = 0; j3 < nv; ++j3) {
                double t0 = 0., t1 = 0., t2 = 0., t3 = 0., t4 = 0.;
                for (int m1 = 0; m1 < 5; ++m1)
                    for (int m2 = 0; m2 < 5; ++m2)
                        for (int m3 = 0; m3 < 5; ++m3) {
                            double x1 = gridv((double)j1) + 0.5 * dv * GX[m1];
                            double x2 = gridv((double)j2) + 0.5 * dv * GX[m2];
                            double x3 = gridv((double)j3) + 0.5 * dv * GX[m3];
                            double fv;
                            if (kind == 0) fv = maxw(x1, x2, x3, 0.9);
                            else if (kind == 1) fv = maxw(x1, x2, x3, 1.0);
                            else fv = 0.5 * (maxw(x1 - u, x2, x3, 1.0) + maxw(x1 + u, x2, x3, 1.0));
                            double tp = GW[m1] * GW[m2] * GW[m3] * fv;
                            t0 += tp;
                            t1 += tp * 0.5 * GX[m1];
                            t2 += tp * 0.5 * GX[m2];
                            t3 += tp * 0.5 * GX[m3];
                            t4 += tp * 0.25 * (GX[m1] * GX[m1] + GX[m2] * GX[m2] + GX[m3] * GX[m3]);
                        }
                t0 = t0 * 0.5 * 0.5 * 0.5; t1 = t1 * 0.5 * 0.5 * 0.5; t2 = t2 * 0.5 * 0.5 * 0.5;
                t3 = t3 * 0.5 * 0.5 * 0.5; t4 = t4 * 0.5 * 0.5 * 0.5;
                for (int i1 = 0; i1 < nx1; ++i1) {
                    const int ig = i1 + i1_off;
                    double sp = std::sin(cw * gridx(ig + 0.5)), sm = std::sin(cw * gridx(ig - 0.5));
                    double tp0 = (dx + (sp - sm) * a / cw) * t0 / dx;
                    double tp5 = (dx + (sp - sm) * a / cw) * t4 / dx;
                    double u1 = (0.5 * (sp + sm) + (std::cos(cw * gridx(ig + 0.5)) - std::cos(cw * gridx(ig - 0.5))) / (cw * dx)) * (a / cw) * t0 * 12. / dx;
                    double u3 = (dx + (sp - sm) * a / cw) * t1 * 12 / dx;
                    double u4 = (dx + (sp - sm) * a / cw) * t2 * 12 / dx;
                    double u5 = (dx + (sp - sm) * a / cw) * t3 * 12 / dx;
                    for (int i2 = 0; i2 < nx2; ++i2) {
                        size_t k = (size_t)i1 * nx2 * T.nv3 + (size_t)i2 * T.nv3 + (j1 * nv * nv + j2 * nv + j3);
                        U[7 * k + 0] = 19 * tp0 / 4. - 15 * tp5;
                        U[7 * k + 6] = 60 * tp5 - 15 * tp0;
                        U[7 * k + 1] = u1;
                        U[7 * k + 3] = u3;
                        U[7 * k + 4] = u4;
                        U[7 * k + 5] = u5;
                    }
                }
            }
}

void destroy(lp_ctx *c) {
    if (!c) return;
    if (c->h2d) { cudaStreamSynchronize(c->h2d); cudaStreamDestroy(c->h2d); }
    if (c->d2h) { cudaStreamSynchronize(c->d2h); cudaStreamDestroy(c->d2h); }
    for (int b = 0; b < 2; ++b) {
        for (int j = 0; j < kHostChunksMax; ++j) {
            if (c->hev_in[b][j]) cudaEventDestroy(c->hev_in[b][j]);
            if (c->hev_col[b][j]) cudaEventDestroy(c->hev_col[b][j]);
        }
        if (c->hev_rest[b]) cudaEventDestroy(c->hev_rest[b]);
        if (c->hev_free[b]) cudaEventDestroy(c->hev_free[b]);
    }
    for (auto &h : c->hgraphs) cudaGraphExecDestroy(h.g);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->cgexec) cudaGraphExecDestroy(c->cgexec);
    if (c->side) { cudaStreamSynchronize(c->side); cudaStreamDestroy(c->side); }
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    for (void *p : c->allocs) cudaFree(p);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

// Context creation.  A batch builds collision-only contexts (one per class
// of runs, over the class's concatenated cells) and advection-only contexts
// (one per run, working on its slice of the class's state buffers).
struct CtxOpts {
    bool collide = true, advect = true;
    double *U = nullptr, *U1 = nullptr, *Ut = nullptr;  // external state buffers
};

lp_status ctx_create(const lp_params *p, const CtxOpts &o, lp_ctx **out) {
    if (!p || !out) return LP_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return LP_ERR_NO_DEVICE;
    }
    lp_ctx *c = new lp_ctx();
    std::string err;
    const unsigned parts = (o.collide ? lp::kTablesCollision : 0u) | (o.advect ? lp::kTablesPoisson : 0u);
    lp_status s = lp::build_tables(*p, c->T, err, parts);
    if (s != LP_OK) {
        delete c;
        return s;
    }
    cudaGetDevice(&c->device);
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess || prop.major != 10 || prop.minor != 3) {
        cudaGetLastError();
        delete c;
        return LP_ERR_NO_DEVICE;
    }
    if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return LP_ERR_CUDA;
    }
    c->stream = c->own_stream;
    c->mixed = (p->precision == LP_PREC_MIXED);
    c->collide_on = o.collide;
    c->advect_on = o.advect;
    c->owns_state = (o.U == nullptr);
    c->Bcap = round32(std::min(std::max(c->T.ncollide, 1), 512));
    c->Bpass = c->Bcap;
    const lp::Tables &T = c->T;
    const size_t rec = (size_t)T.size * 7;
    if (o.collide) s = c->mixed ? upload_tables<float>(c) : upload_tables<double>(c);
    if (s == LP_OK && c->LW &&
        (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
         cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess))
        s = LP_ERR_CUDA;
    if (s == LP_OK && c->owns_state) {
        s = dalloc(c, &c->U, rec);
        if (s == LP_OK) s = dalloc(c, &c->U1, rec);
        if (s == LP_OK) s = dalloc(c, &c->Ut, rec);
    } else if (s == LP_OK) {
        c->U = o.U; c->U1 = o.U1; c->Ut = o.Ut;
    }
    if (s == LP_OK && o.advect) s = setup_advection(c);
    if (s == LP_OK) s = dalloc(c, &c->mpart, 5 * kMomBlocks);
    if (s == LP_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) s = LP_ERR_CUDA;
    if (s != LP_OK) {
        fprintf(stderr, "lp_ctx_create: %s\n", c->err.c_str());
        destroy(c);
        return s;
    }
    *out = c;
    return LP_OK;
}

// ============================================================== adjoint
// Vector-Jacobian products of the FP64 path (see lp_adjoint.cu for the
// conventions), evaluated at given states; every forward quantity they need
// is recomputed from the state.

lp_status adj_setup(lp_ctx *c) {
    auto &A = c->adj;
    if (A.ready) return LP_OK;
    const lp::Tables &T = c->T;
    if (c->mixed || !c->collide_on || !c->advect_on) return fail(c, LP_ERR_INVALID, "the adjoint needs an FP64 context");
    if (c->WLin) return fail(c, LP_ERR_INVALID, "the adjoint covers the one-species operator");
    if ((T.prm.fixes & (LP_FIX_F1 | LP_FIX_F2 | LP_FIX_F3)) != (LP_FIX_F1 | LP_FIX_F2 | LP_FIX_F3))
        return fail(c, LP_ERR_INVALID, "the adjoint needs LP_FIX_F1 | LP_FIX_F2 | LP_FIX_F3");
    if (T.pois.ndim > 4096) return fail(c, LP_ERR_INVALID, "the adjoint needs a Poisson matrix of order <= 4096");
    const size_t n3 = T.n3, Bp = c->Bcap, rec = (size_t)T.size * 7, nc = T.ncell;
    for (int s = 0; s < 4; ++s) LP_TRY(dalloc(c, &A.F[s], n3 * Bp));
    LP_TRY(dalloc(c, &A.r1, n3 * Bp));
    LP_TRY(dalloc(c, &A.r2, n3 * Bp));
    LP_TRY(dalloc(c, &A.lf, n3 * Bp));
    LP_TRY(dalloc(c, &A.lqn, n3 * Bp));
    LP_TRY(dalloc(c, &A.ls, n3 * Bp));
    LP_TRY(dalloc(c, &A.ltp, 5 * (size_t)T.nv3 * Bp));
    LP_TRY(dalloc(c, &A.lq, n3 * Bp));
    LP_TRY(dalloc(c, &A.tq, n3 * Bp));
    LP_TRY(dalloc(c, &A.lF, n3 * Bp));
    LP_TRY(dalloc(c, &A.qs, n3 * Bp));
    // conjugate transposes of the per-axis matrices (out index major)
    std::vector<double> fH(T.mfwd.size()), iH(T.minv.size());
    const int n = T.n;
    for (int p = 0; p < n; ++p)
        for (int a = 0; a < n; ++a) {
            fH[2 * (a * n + p)] = T.mfwd[2 * (p * n + a)];
            fH[2 * (a * n + p) + 1] = -T.mfwd[2 * (p * n + a) + 1];
            iH[2 * (a * n + p)] = T.minv[2 * (p * n + a)];
            iH[2 * (a * n + p) + 1] = -T.minv[2 * (p * n + a) + 1];
        }
    LP_TRY(upload(c, &A.mfH, fH.data(), fH.size()));
    LP_TRY(upload(c, &A.miH, iH.data(), iH.size()));
    // spectral nodes inside each DG velocity cell (nodecell is nondecreasing)
    std::vector<int> first(T.nv, 0), count(T.nv, 0);
    for (int l = n - 1; l >= 0; --l) { first[T.nodecell[l]] = l; ++count[T.nodecell[l]]; }
    LP_TRY(upload(c, &A.nfirst, first.data(), first.size()));
    LP_TRY(upload(c, &A.ncount, count.data(), count.size()));
    std::vector<double> inv;
    lp::poisson_inverse(T.pois, inv);
    LP_TRY(upload(c, &A.Ainv, inv.data(), inv.size()));
    LP_TRY(dalloc(c, &A.lrt, 3 * nc));
    LP_TRY(dalloc(c, &A.lamF, 3 * nc));
    LP_TRY(dalloc(c, &A.lphix, 3 * nc));
    LP_TRY(dalloc(c, &A.lphiy, 3 * nc));
    LP_TRY(dalloc(c, &A.J, 1));
    LP_TRY(dalloc(c, &A.dnu, (size_t)std::max(T.ncollide, 1)));
    LP_TRY(dalloc(c, &A.lU, rec));
    LP_TRY(dalloc(c, &A.lU1, rec));
    LP_TRY(dalloc(c, &A.lUt, rec));
    LP_TRY(dalloc(c, &A.lH, rec));
    LP_TRY(dalloc(c, &A.lC, rec));
    LP_TRY(dalloc(c, &A.Ukeep, rec));
    {
        std::vector<double> Cp, Wf, Wi;
        lp::corr_tables(T.shat.data(), T.ahat.data(), T.cw.data(), T.h_eta, n, Cp, Wf, Wi);
        LP_TRY(upload(c, &A.Cp, Cp.data(), Cp.size()));
        double *wf = nullptr, *wi = nullptr;
        LP_TRY(upload(c, &wf, Wf.data(), Wf.size()));
        LP_TRY(upload(c, &wi, Wi.data(), Wi.size()));
        A.Wf = reinterpret_cast<double2 *>(wf);
        A.Wi = reinterpret_cast<double2 *>(wi);
        LP_TRY(dalloc(c, &A.cscr, lp::corr_scratch_elems(n)));
    }
    A.ready = true;
    return LP_OK;
}

// q = conserve(ComputeQ(F)) for the FP64 pair table
lp_status adj_q(lp_ctx *c, const double2 *F, int Bp, double2 *q) {
    const lp::Tables &T = c->T;
    LP_CUDA(lp::launch_computeq<double>(F, (const double *)c->P, c->PI, c->pair_off, T.n3, Bp, q, c->stream));
    LP_CUDA(lp::launch_conserve(q, c->c1, c->c2, c->cct, T.n3, Bp, c->cpart, c->nchunk, c->lam, c->stream));
    return LP_OK;
}

// lam_f_out (=|+=) Re T^H conserve(lam_q) through the linearised ComputeQ at F
lp_status adj_q_back(lp_ctx *c, const double2 *F, double2 *lq, int Bp, double *lf, double beta) {
    const lp::Tables &T = c->T;
    auto &A = c->adj;
    const long long N = (long long)T.n3 * Bp;
    LP_CUDA(lp::launch_conserve(lq, c->c1, c->c2, c->cct, T.n3, Bp, c->cpart, c->nchunk, c->lam, c->stream));
    if (A.qvjp_form == 0)
        LP_CUDA(lp::launch_qvjp_corr(F, lq, A.Cp, A.Wf, A.Wi, T.n, Bp, Bp, A.lF, A.cscr, c->stream));
    else
        LP_CUDA(lp::launch_qvjp(F, lq, (const double *)c->P, c->pair_off, T.n, Bp, A.lF, c->stream));
    LP_CUDA(lp::launch_fwd_complex<double>(A.lF, (double2 *)c->t1, A.tq, A.mfH, T.n, Bp, c->stream));
    LP_CUDA(lp::launch_add_re(lf, beta, A.tq, 1.0, N, c->stream));
    return LP_OK;
}

// lam_in = (d collision step / dU at Uin)^T lam_out for cells [0, ncollide);
// dnu[cell] += the cell's dL/dnu.  Uin is the collision's input state.
lp_status collide_vjp(lp_ctx *c, const double *Uin, const double *lout, double *lin) {
    LP_TRY(adj_setup(c));
    auto &A = c->adj;
    const lp::Tables &T = c->T;
    const double dt = T.prm.dt, nu = T.prm.nu;
    const double kfac = 1. / T.scalev / T.scaleL / T.scale3;
    // records of cells that are not collided keep their adjoint
    LP_CUDA(cudaMemcpyAsync(lin, lout, sizeof(double) * (size_t)T.size * 7, cudaMemcpyDeviceToDevice, c->stream));
    LP_CUDA(cudaMemsetAsync(A.dnu, 0, sizeof(double) * std::max(T.ncollide, 1), c->stream));
    if (!(nu > 0.)) return LP_OK;
    const double *Mf = (const double *)c->mfwd, *Mi = (const double *)c->minv;
    double *f = (double *)c->f, *f1 = (double *)c->f1, *qn = (double *)c->qn;
    for (int c0 = 0; c0 < T.ncollide; c0 += c->Bcap) {
        const int B = std::min(c->Bcap, T.ncollide - c0), Bp = round32(B);
        const long long N = (long long)T.n3 * Bp;
        double2 *t1 = (double2 *)c->t1, *t2 = (double2 *)c->t2, *tc = (double2 *)c->Qc;
        // forward recomputation of the stages
        LP_CUDA(lp::launch_nodes<double>(Uin, T.nv, T.n, c0, B, Bp, 3, c->nodecell, c->nodeoff, T.dv, f, c->stream));
        LP_CUDA(lp::launch_fwd<double>(f, t1, A.F[0], Mf, T.n, Bp, c->stream));
        LP_TRY(adj_q(c, A.F[0], Bp, c->q[0]));
        LP_CUDA(lp::launch_fs_full<double>(c->q[0], t1, t2, tc, Mi, T.n, Bp, c->stream));
        LP_CUDA(lp::launch_add_re(qn, 0., tc, 1., N, c->stream));                  // qn = Re FS(q0)
        LP_CUDA(cudaMemcpyAsync(f1, f, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
        LP_CUDA(lp::launch_axpby(f1, 1., qn, dt * nu, N, c->stream));                // f + dt nu qn
        LP_CUDA(lp::launch_fwd<double>(f1, t1, A.F[1], Mf, T.n, Bp, c->stream));
        LP_TRY(adj_q(c, A.F[1], Bp, c->q[1]));
        double *rs[2] = {A.r1, A.r2};
        for (int s = 1; s <= 2; ++s) {
            LP_CUDA(lp::launch_fs_full<double>(c->q[s], t1, t2, tc, Mi, T.n, Bp, c->stream));
            LP_CUDA(lp::launch_add_re(rs[s - 1], 0., tc, 1., N, c->stream));       // r_s = Re FS(q_s)
            LP_CUDA(cudaMemcpyAsync(f1, f, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
            LP_CUDA(lp::launch_axpby(f1, 1., qn, 0.5 * dt * nu, N, c->stream));
            LP_CUDA(lp::launch_axpby(f1, 1., rs[s - 1], 0.5 * dt * nu, N, c->stream));
            LP_CUDA(lp::launch_fwd<double>(f1, t1, A.F[s + 1], Mf, T.n, Bp, c->stream));
            LP_TRY(adj_q(c, A.F[s + 1], Bp, c->q[s + 1]));
        }
        // backward: the update of the collided coefficients and the projection
        LP_CUDA(lp::launch_collide_out_vjp(lout, T.nv, c0, B, Bp, dt, kfac, A.ltp, lin, c->stream));
        LP_CUDA(lp::launch_project_vjp(A.ltp, (const double *)c->tfac, T.n, T.nv, Bp, (double2 *)c->Z,
                                       (double2 *)c->Y, tc, c->stream));           // tc = lam_Qc
        LP_CUDA(lp::launch_qsum(c->q[0], c->q[1], c->q[2], c->q[3], N, A.qs, c->stream));
        LP_CUDA(lp::launch_cdot_cell(tc, A.qs, T.n3, Bp, B, 1.0, A.dnu + c0, c->stream));
        // q3 <- F3 <- f1_2 = f + dt nu/2 (qn + r2)
        LP_CUDA(lp::launch_caxpby(A.lq, 0., tc, nu / 6., N, c->stream));
        LP_TRY(adj_q_back(c, A.F[3], A.lq, Bp, A.ls, 0.));                       // ls = lam f1_2
        LP_CUDA(cudaMemcpyAsync(A.lf, A.ls, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
        LP_CUDA(lp::launch_scale(A.lqn, A.ls, 0.5 * dt * nu, N, c->stream));
        LP_CUDA(lp::launch_dot_cell(A.ls, qn, T.n3, Bp, B, 0.5 * dt, A.dnu + c0, c->stream));
        LP_CUDA(lp::launch_dot_cell(A.ls, A.r2, T.n3, Bp, B, 0.5 * dt, A.dnu + c0, c->stream));
        for (int s = 2; s >= 1; --s) {
            // lam q_s = nu/6 lam_Qc + FS^H (dt nu/2 lam f1_s)
            LP_CUDA(lp::launch_fwd<double>(A.ls, t1, A.lq, A.miH, T.n, Bp, c->stream));
            LP_CUDA(lp::launch_caxpby(A.lq, 0.5 * dt * nu, tc, nu / 6., N, c->stream));
            LP_TRY(adj_q_back(c, A.F[s], A.lq, Bp, A.ls, 0.));                   // ls = lam f1_{s-1}
            LP_CUDA(lp::launch_axpby(A.lf, 1., A.ls, 1., N, c->stream));
            if (s == 2) {  // f1_1 = f + dt nu/2 (qn + r1)
                LP_CUDA(lp::launch_axpby(A.lqn, 1., A.ls, 0.5 * dt * nu, N, c->stream));
                LP_CUDA(lp::launch_dot_cell(A.ls, qn, T.n3, Bp, B, 0.5 * dt, A.dnu + c0, c->stream));
                LP_CUDA(lp::launch_dot_cell(A.ls, A.r1, T.n3, Bp, B, 0.5 * dt, A.dnu + c0, c->stream));
            } else {       // f1_0 = f + dt nu qn
                LP_CUDA(lp::launch_axpby(A.lqn, 1., A.ls, dt * nu, N, c->stream));
                LP_CUDA(lp::launch_dot_cell(A.ls, qn, T.n3, Bp, B, dt, A.dnu + c0, c->stream));
            }
        }
        // q0: nu/2 lam_Qc + FS^H lam_qn
        LP_CUDA(lp::launch_fwd<double>(A.lqn, t1, A.lq, A.miH, T.n, Bp, c->stream));
        LP_CUDA(lp::launch_caxpby(A.lq, 1., tc, nu / 2., N, c->stream));
        LP_TRY(adj_q_back(c, A.F[0], A.lq, Bp, A.lf, 1.));
        LP_CUDA(lp::launch_nodes_vjp(A.lf, T.nv, T.n, c0, B, Bp, 3, A.nfirst, A.ncount, c->nodeoff, lin, c->stream));
    }
    return LP_OK;
}

// lam (accumulated) += (d/dV of dt-scaled flux stage)^T: lamV += (dH/dV)^T lamH
// with the Poisson solve of V included.
lp_status flux_stage_vjp(lp_ctx *c, const double *V, const double *lamH, double *lamV) {
    auto &A = c->adj;
    const lp::Tables &T = c->T;
    LP_TRY(poisson_on(c, V));  // fields of V
    LP_CUDA(cudaMemsetAsync(A.lamF, 0, sizeof(double) * 3 * T.ncell, c->stream));
    LP_CUDA(lp::launch_flux_vjp(advect_dev(c), V, c->fields, lamH, lamV, A.lamF, c->stream));
    LP_CUDA(lp::launch_poisson_vjp(poisson_dev(c, false), A.lamF, nullptr, nullptr, A.Ainv, A.lrt, c->stream));
    LP_CUDA(lp::launch_charge_vjp(A.lrt, T.size, T.nv3, T.scalev, lamV, c->stream));
    return LP_OK;
}

// lam_in = (d RK3 step / dU at U)^T lam_out, with U1, Ut the step's stage
// values (recomputed by the caller).
lp_status advect_vjp(lp_ctx *c, const double *U, const double *U1, const double *Ut, const double *lout,
                     double *lin) {
    auto &A = c->adj;
    const lp::Tables &T = c->T;
    const long long n = (long long)T.size * 7;
    const double dt = T.prm.dt;
    // U_new = U/3 + 2/3 Ut + 2/3 dt H(Ut)
    LP_CUDA(lp::launch_scale(lin, lout, 1. / 3., n, c->stream));
    LP_CUDA(lp::launch_scale(A.lUt, lout, 2. / 3., n, c->stream));
    LP_CUDA(lp::launch_scale(A.lH, lout, 2. / 3. * dt, n, c->stream));
    LP_TRY(flux_stage_vjp(c, Ut, A.lH, A.lUt));
    // Ut = 3/4 U + 1/4 U1 + 1/4 dt H(U1)
    LP_CUDA(lp::launch_axpby(lin, 1., A.lUt, 0.75, n, c->stream));
    LP_CUDA(lp::launch_scale(A.lU1, A.lUt, 0.25, n, c->stream));
    LP_CUDA(lp::launch_scale(A.lH, A.lUt, 0.25 * dt, n, c->stream));
    LP_TRY(flux_stage_vjp(c, U1, A.lH, A.lU1));
    // U1 = U + dt H(U)
    LP_CUDA(lp::launch_axpby(lin, 1., A.lU1, 1., n, c->stream));
    LP_CUDA(lp::launch_scale(A.lH, A.lU1, dt, n, c->stream));
    LP_TRY(flux_stage_vjp(c, U, A.lH, lin));
    return LP_OK;
}

// Field energy J of state U (device) and, if lamU, dJ/dU into lamU.
lp_status field_energy_at(lp_ctx *c, const double *U, double *lamU) {
    auto &A = c->adj;
    const lp::Tables &T = c->T;
    LP_TRY(poisson_on(c, U));
    LP_CUDA(lp::launch_field_energy(c->phix, c->phiy, T.ncell, T.dx * T.dy, A.J, A.lphix, A.lphiy, c->stream));
    if (lamU) {
        LP_CUDA(cudaMemsetAsync(lamU, 0, sizeof(double) * (size_t)T.size * 7, c->stream));
        LP_CUDA(lp::launch_poisson_vjp(poisson_dev(c, false), nullptr, A.lphix, A.lphiy, A.Ainv, A.lrt, c->stream));
        LP_CUDA(lp::launch_charge_vjp(A.lrt, T.size, T.nv3, T.scalev, lamU, c->stream));
    }
    return LP_OK;
}

// One time step's VJP at state Un (device, not c->U): lam <- (dStep/dU)^T lam,
// adding the step's dL/dnu to *dnu_sum.  Uses c->U, U1, Ut as scratch.
lp_status step_vjp(lp_ctx *c, const double *Un, double *lam, double *dnu_sum) {
    auto &A = c->adj;
    const lp::Tables &T = c->T;
    const size_t bytes = sizeof(double) * (size_t)T.size * 7;
    LP_CUDA(cudaMemcpyAsync(c->U, Un, bytes, cudaMemcpyDeviceToDevice, c->stream));
    LP_TRY(advect(c));  // c->U = advected state, c->U1, c->Ut = stage values
    LP_TRY(collide_vjp(c, c->U, lam, A.lC));
    if (dnu_sum) {
        std::vector<double> d(std::max(T.ncollide, 1));
        LP_CUDA(cudaMemcpyAsync(d.data(), A.dnu, sizeof(double) * d.size(), cudaMemcpyDeviceToHost, c->stream));
        LP_CUDA(cudaStreamSynchronize(c->stream));
        if (T.prm.nu > 0.)
            for (int i = 0; i < T.ncollide; ++i) *dnu_sum += d[i];
    }
    LP_TRY(advect_vjp(c, Un, c->U1, c->Ut, A.lC, lam));
    return LP_OK;
}

}  // namespace

extern "C" {

lp_status lp_ctx_create(const lp_params *p, lp_ctx **out) { return ctx_create(p, CtxOpts{}, out); }

lp_status lp_ctx_destroy(lp_ctx *c) {
    if (!c) return LP_ERR_INVALID;
    cudaStreamSynchronize(c->stream);
    destroy(c);
    return LP_OK;
}

lp_status lp_set_stream(lp_ctx *c, void *st) {
    if (!c) return LP_ERR_INVALID;
    c->stream = st ? (cudaStream_t)st : c->own_stream;
    return LP_OK;
}

lp_status lp_synchronize(lp_ctx *c) {
    if (!c) return LP_ERR_INVALID;
    LP_CUDA(cudaStreamSynchronize(c->stream));
    if (c->h2d) LP_CUDA(cudaStreamSynchronize(c->h2d));
    if (c->d2h) LP_CUDA(cudaStreamSynchronize(c->d2h));
    if (c->tc_err) {  // a bounded wait of the tensor-core projection or the fused convolution that ran out
        int e = 0;
        LP_CUDA(cudaMemcpy(&e, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (e) return fail(c, LP_ERR_CUDA, std::string(e >= 3 ? "fused convolution" : "tensor-core projection") +
                                               ": a bounded wait ran out (code " + std::to_string(e) + ")");
    }
    return LP_OK;
}

const char *lp_last_error(const lp_ctx *c) { return c ? c->err.c_str() : "null context"; }

size_t lp_device_bytes(const lp_ctx *c) { return c ? c->bytes : 0; }

lp_status lp_set_state(lp_ctx *c, const double *U, size_t n) {
    if (!c || !U || n != (size_t)c->T.size * 7) return fail(c, LP_ERR_INVALID, "state size mismatch");
    LP_CUDA(cudaMemcpyAsync(c->U, U, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    c->has_state = true;
    return LP_OK;
}

lp_status lp_get_state(lp_ctx *c, double *U, size_t n) {
    if (!c || !U || n != (size_t)c->T.size * 7) return fail(c, LP_ERR_INVALID, "state size mismatch");
    LP_CUDA(cudaMemcpyAsync(U, c->U, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}

lp_status lp_state_device_ptr(lp_ctx *c, double **U) {
    if (!c || !U) return LP_ERR_INVALID;
    *U = c->U;
    c->has_state = true;
    return LP_OK;
}

lp_status lp_set_init(lp_ctx *c, int kind, double u) {
    if (!c || kind < 0 || kind > 2) return fail(c, LP_ERR_INVALID, "unknown initial condition");
    std::vector<double> U;
    set_init_host(c->T, kind, u, U, c->i1_off);
    return lp_set_state(c, U.data(), U.size());
}

lp_status lp_fft3d(lp_ctx *c, const double *in, double *out) {
    if (!c || !in || !out) return LP_ERR_INVALID;
    return c->mixed ? do_fft3d<float>(c, in, out, false) : do_fft3d<double>(c, in, out, false);
}

lp_status lp_fs(lp_ctx *c, const double *in, double *out) {
    if (!c || !in || !out) return LP_ERR_INVALID;
    return c->mixed ? do_fft3d<float>(c, in, out, true) : do_fft3d<double>(c, in, out, true);
}

lp_status lp_compute_q(lp_ctx *c, const double *f, double *qhat) {
    if (!c || !f || !qhat) return LP_ERR_INVALID;
    return c->mixed ? do_compute_q<float>(c, f, qhat) : do_compute_q<double>(c, f, qhat);
}

lp_status lp_conserve(lp_ctx *c, double *qhat) {
    if (!c || !qhat) return LP_ERR_INVALID;
    const lp::Tables &T = c->T;
    LP_TRY(put_cplx_column<double>(c, c->q[0], qhat, T.n3));
    LP_CUDA(lp::launch_conserve(c->q[0], c->c1, c->c2, c->cct, T.n3, 32, c->cpart, c->nchunk, c->lam, c->stream));
    return get_cplx_column<double>(c, qhat, c->q[0], T.n3);
}

lp_status lp_rk4_cell(lp_ctx *c, const double *f, int cell, const double *qhat, double *dU) {
    if (!c || !f || !qhat || !dU || cell < 0 || cell >= c->T.ncell) return fail(c, LP_ERR_INVALID, "bad argument");
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    return c->mixed ? do_rk4_cell<float>(c, f, cell, qhat, dU) : do_rk4_cell<double>(c, f, cell, qhat, dU);
}

lp_status lp_compute_q_lin(lp_ctx *c, const double *f, double *qhat, double *qhat_lin) {
    if (!c || !f || !qhat || !qhat_lin) return LP_ERR_INVALID;
    if (!c->WLin) return fail(c, LP_ERR_INVALID, "not a two-species context");
    return c->mixed ? do_compute_q<float>(c, f, qhat, qhat_lin) : do_compute_q<double>(c, f, qhat, qhat_lin);
}

lp_status lp_conserve_lin(lp_ctx *c, double *qhat, double *qhat_lin) {
    if (!c || !qhat || !qhat_lin) return LP_ERR_INVALID;
    if (!c->WLin) return fail(c, LP_ERR_INVALID, "not a two-species context");
    const lp::Tables &T = c->T;
    LP_TRY(put_cplx_column<double>(c, c->q[0], qhat, T.n3));
    LP_TRY(put_cplx_column<double>(c, c->qlin, qhat_lin, T.n3));
    LP_CUDA(lp::launch_conserve(c->q[0], c->c1, c->c2, c->cct, T.n3, 32, c->cpart, c->nchunk, c->lam, c->stream));
    LP_CUDA(lp::launch_conserve(c->qlin, c->c1, c->c2, c->cct_lin5, T.n3, 32, c->cpart, c->nchunk, c->lam,
                                c->stream));
    LP_TRY(get_cplx_column<double>(c, qhat, c->q[0], T.n3));
    return get_cplx_column<double>(c, qhat_lin, c->qlin, T.n3);
}

lp_status lp_rk4_cell_lin(lp_ctx *c, const double *f, int cell, const double *qhat, const double *qhat_lin,
                          double *dU) {
    if (!c || !f || !qhat || !qhat_lin || !dU || cell < 0 || cell >= c->T.ncell)
        return fail(c, LP_ERR_INVALID, "bad argument");
    if (!c->WLin) return fail(c, LP_ERR_INVALID, "not a two-species context");
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    // the two-species RK4 starts from qHat + qHat_linear (C:644-648)
    std::vector<double> q0(2 * (size_t)c->T.n3);
    for (size_t i = 0; i < q0.size(); ++i) q0[i] = qhat[i] + qhat_lin[i];
    return c->mixed ? do_rk4_cell<float>(c, f, cell, q0.data(), dU) : do_rk4_cell<double>(c, f, cell, q0.data(), dU);
}

lp_status lp_nodes(lp_ctx *c, double *f) {
    if (!c || !f) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    const lp::Tables &T = c->T;
    const int slot1 = (T.prm.fixes & LP_FIX_F2) ? 3 : 2;
    double *tmp = (double *)c->q[0];  // n3 * Bcap doubles fit in a complex buffer
    for (int b0 = 0; b0 < T.ncollide; b0 += c->Bcap) {
        const int B = std::min(c->Bcap, T.ncollide - b0), Bp = round32(B);
        LP_CUDA(lp::launch_nodes<double>(c->U, T.nv, T.n, b0, B, Bp, slot1, c->nodecell, c->nodeoff, T.dv, tmp,
                                         c->stream));
        for (int cc = 0; cc < B; ++cc)
            LP_CUDA(cudaMemcpy2DAsync(f + (size_t)(b0 + cc) * T.n3, sizeof(double), tmp + cc, sizeof(double) * Bp,
                                      sizeof(double), T.n3, cudaMemcpyDeviceToHost, c->stream));
        LP_CUDA(cudaStreamSynchronize(c->stream));
    }
    return LP_OK;
}

lp_status lp_weights_rows(lp_ctx *c, int r0, int r1, double *out) {
    if (!c || !out || r0 < 0 || r1 > c->T.n3 || r0 > r1) return fail(c, LP_ERR_INVALID, "bad row range");
    for (int r = r0; r < r1; ++r)
        for (int o = 0; o < c->T.n3; ++o) out[(size_t)(r - r0) * c->T.n3 + o] = lp::weight_host(c->T, r, o);
    return LP_OK;
}

lp_status lp_conservation_rows(lp_ctx *c, double *c1, double *c2, double *cct) {
    if (!c) return LP_ERR_INVALID;
    if (c1) std::memcpy(c1, c->T.c1.data(), sizeof(double) * c->T.c1.size());
    if (c2) std::memcpy(c2, c->T.c2.data(), sizeof(double) * c->T.c2.size());
    if (cct) std::memcpy(cct, c->T.cct_inv, sizeof(double) * 25);
    return LP_OK;
}

lp_status lp_poisson(lp_ctx *c, double *potc, double *phix, double *phiy, double *fields) {
    if (!c) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    LP_TRY(poisson_on(c, c->U));
    const size_t nc = c->T.ncell;
    if (potc) LP_CUDA(cudaMemcpyAsync(potc, c->potc, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream));
    if (phix) LP_CUDA(cudaMemcpyAsync(phix, c->phix, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream));
    if (phiy) LP_CUDA(cudaMemcpyAsync(phiy, c->phiy, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream));
    if (fields) LP_CUDA(cudaMemcpyAsync(fields, c->fields, sizeof(double) * 14 * nc, cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}

lp_status lp_last_fields(lp_ctx *c, double *potc, double *phix, double *phiy, double *fields) {
    if (!c) return LP_ERR_INVALID;
    const size_t nc = c->T.ncell;
    if (potc) LP_CUDA(cudaMemcpyAsync(potc, c->potc, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream));
    if (phix) LP_CUDA(cudaMemcpyAsync(phix, c->phix, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream));
    if (phiy) LP_CUDA(cudaMemcpyAsync(phiy, c->phiy, sizeof(double) * 3 * nc, cudaMemcpyDeviceToHost, c->stream));
    if (fields) LP_CUDA(cudaMemcpyAsync(fields, c->fields, sizeof(double) * 14 * nc, cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}

lp_status lp_advect_step(lp_ctx *c) {
    if (!c) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    return advect(c);
}

lp_status lp_collision_step(lp_ctx *c, int cell_begin, int cell_end) {
    NvtxRange r("lp_collision_step");
    if (!c) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    if (cell_begin == -1 && cell_end == -1) { cell_begin = 0; cell_end = c->T.ncollide; }
    if (cell_begin < 0 || cell_end > c->T.ncollide || cell_begin > cell_end)
        return fail(c, LP_ERR_INVALID, "bad cell range");
    if (cell_begin != 0 || cell_end != c->T.ncollide || cell_end == 0) return collide(c, cell_begin, cell_end);
    // all collided cells: one captured graph, replayed
    if (!c->cgexec || c->cgstream != c->stream) {
        if (c->cgexec) { cudaGraphExecDestroy(c->cgexec); c->cgexec = nullptr; }
        cudaGraph_t g = nullptr;
        LP_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        lp_status s = collide(c, 0, c->T.ncollide);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (s != LP_OK) { if (g) cudaGraphDestroy(g); return s; }
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
        size_t nn = 0;
        c->cg_kernels = 0;
        if (cudaGraphGetNodes(g, nullptr, &nn) == cudaSuccess && nn) {
            std::vector<cudaGraphNode_t> nodes(nn);
            if (cudaGraphGetNodes(g, nodes.data(), &nn) == cudaSuccess)
                for (size_t i = 0; i < nn; ++i) {
                    cudaGraphNodeType ty;
                    if (cudaGraphNodeGetType(nodes[i], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel)
                        ++c->cg_kernels;
                }
        }
        e = instantiate_step_graph(&c->cgexec, g, &c->cg_pdl);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
        c->cgstream = c->stream;
    }
    LP_CUDA(cudaGraphLaunch(c->cgexec, c->stream));
    return LP_OK;
}

lp_status lp_collision_step_host(lp_ctx *c, const double *U_in, double *U_out, int chunks, int flags) {
    NvtxRange r("lp_collision_step_host");
    if (!c || !U_in || !U_out || chunks < 1 || chunks > kHostChunksMax || (flags & ~LP_HOST_ASYNC))
        return LP_ERR_INVALID;
    if (!c->collide_on || !c->owns_state) return fail(c, LP_ERR_INVALID, "no collision tables or state in this context");
    const lp::Tables &T = c->T;
    if (chunks > 1 && !(T.prm.fixes & LP_FIX_F1))
        return fail(c, LP_ERR_INVALID, "reference slot reads (F1 unfixed) need all cells in one chunk");
    const size_t rec = (size_t)T.nv3 * 7;  // doubles per spatial cell
    if (!c->h2d) {
        LP_TRY(dalloc(c, &c->hstage[0], rec * T.ncell));
        LP_TRY(dalloc(c, &c->hstage[1], rec * T.ncell));
        LP_CUDA(cudaStreamCreateWithFlags(&c->h2d, cudaStreamNonBlocking));
        LP_CUDA(cudaStreamCreateWithFlags(&c->d2h, cudaStreamNonBlocking));
        for (int b = 0; b < 2; ++b) {
            for (int j = 0; j < kHostChunksMax; ++j) {
                LP_CUDA(cudaEventCreateWithFlags(&c->hev_in[b][j], cudaEventDisableTiming));
                LP_CUDA(cudaEventCreateWithFlags(&c->hev_col[b][j], cudaEventDisableTiming));
            }
            LP_CUDA(cudaEventCreateWithFlags(&c->hev_rest[b], cudaEventDisableTiming));
            LP_CUDA(cudaEventCreateWithFlags(&c->hev_free[b], cudaEventDisableTiming));
            LP_CUDA(cudaEventRecord(c->hev_free[b], c->d2h));
        }
    }
    const int ncol = T.ncollide, ncell = T.ncell;
    const int per = std::max(32, round32((ncol + chunks - 1) / chunks));
    const int b = c->hnext;
    c->hnext ^= 1;
    double *Us = c->hstage[b];
    // the copies into staging state b start once its last copy out is done:
    // the previous call's collision (on the other staging state) can still run
    LP_CUDA(cudaStreamWaitEvent(c->h2d, c->hev_free[b], 0));
    int nch = 0;
    for (int c0 = 0; c0 < ncol; c0 += per, ++nch) {
        const int c1 = std::min(ncol, c0 + per);
        LP_CUDA(cudaMemcpyAsync(Us + c0 * rec, U_in + c0 * rec, sizeof(double) * rec * (c1 - c0),
                                cudaMemcpyHostToDevice, c->h2d));
        LP_CUDA(cudaEventRecord(c->hev_in[b][nch], c->h2d));
    }
    if (ncell > ncol) {  // cells that are not collided pass through unchanged
        LP_CUDA(cudaMemcpyAsync(Us + ncol * rec, U_in + ncol * rec, sizeof(double) * rec * (ncell - ncol),
                                cudaMemcpyHostToDevice, c->h2d));
        LP_CUDA(cudaEventRecord(c->hev_rest[b], c->h2d));
    }
    // chunk j collides (a captured graph per staging state and cell range, on
    // the context's stream) once its records are on the device, and is copied
    // back while chunk j + 1 collides
    int j = 0;
    for (int c0 = 0; c0 < ncol; c0 += per, ++j) {
        const int c1 = std::min(ncol, c0 + per);
        cudaGraphExec_t g = nullptr;
        for (auto &h : c->hgraphs)
            if (h.b == b && h.c0 == c0 && h.c1 == c1) g = h.g;
        if (!g) {
            double *keep = c->U;
            c->U = Us;  // the captured kernels take the staging state
            cudaGraph_t gr = nullptr;
            LP_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            lp_status st = collide(c, c0, c1);
            cudaError_t e = cudaStreamEndCapture(c->stream, &gr);
            c->U = keep;
            if (st != LP_OK) { if (gr) cudaGraphDestroy(gr); return st; }
            if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
            e = instantiate_step_graph(&g, gr);
            cudaGraphDestroy(gr);
            if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
            c->hgraphs.push_back({b, c0, c1, g});
        }
        LP_CUDA(cudaStreamWaitEvent(c->stream, c->hev_in[b][j], 0));
        LP_CUDA(cudaGraphLaunch(g, c->stream));
        LP_CUDA(cudaEventRecord(c->hev_col[b][j], c->stream));
        LP_CUDA(cudaStreamWaitEvent(c->d2h, c->hev_col[b][j], 0));
        LP_CUDA(cudaMemcpyAsync(U_out + c0 * rec, Us + c0 * rec, sizeof(double) * rec * (c1 - c0),
                                cudaMemcpyDeviceToHost, c->d2h));
    }
    if (ncell > ncol) {
        LP_CUDA(cudaStreamWaitEvent(c->d2h, c->hev_rest[b], 0));
        LP_CUDA(cudaMemcpyAsync(U_out + ncol * rec, Us + ncol * rec, sizeof(double) * rec * (ncell - ncol),
                                cudaMemcpyDeviceToHost, c->d2h));
    }
    LP_CUDA(cudaEventRecord(c->hev_free[b], c->d2h));
    // without LP_HOST_ASYNC the context's stream orders after the last copy
    if (!(flags & LP_HOST_ASYNC)) LP_CUDA(cudaStreamWaitEvent(c->stream, c->hev_free[b], 0));
    return LP_OK;
}

lp_status lp_collision_graph_kernels(lp_ctx *c, int *kernels) {
    if (!c || !kernels) return LP_ERR_INVALID;
    *kernels = c->cgexec ? c->cg_kernels : 0;
    return LP_OK;
}

lp_status lp_collision_graph_edges(lp_ctx *c, int *programmatic) {
    if (!c || !programmatic) return LP_ERR_INVALID;
    *programmatic = c->cgexec ? c->cg_pdl : 0;
    return LP_OK;
}

lp_status lp_step(lp_ctx *c, int nsteps) {
    NvtxRange r("lp_step");
    if (!c || nsteps < 0) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    if (nsteps == 0) return LP_OK;
    if (!c->gexec || c->gstream != c->stream) {
        if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
        cudaGraph_t g = nullptr;
        LP_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        lp_status s = one_step(c);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (s != LP_OK) { if (g) cudaGraphDestroy(g); return s; }
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
        e = instantiate_step_graph(&c->gexec, g);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
        c->gstream = c->stream;
    }
    for (int i = 0; i < nsteps; ++i) LP_CUDA(cudaGraphLaunch(c->gexec, c->stream));
    return LP_OK;
}

lp_status lp_time_kernel(lp_ctx *c, int which, int reps, double *ms) {
    if (!c || !ms || reps < 1 || which < 0 || which > 8) return fail(c, LP_ERR_INVALID, "bad argument");
    if (which >= 4 && !(c->FQC && c->line_warps == 0))
        return fail(c, LP_ERR_INVALID, "the convolution form is not this context's schedule");
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    const lp::Tables &T = c->T;
    const int B = std::min(c->Bcap, T.ncollide), Bp = round32(B);
    // inputs of every stage: node values, transform, one conserved mode array
    lp_status s = c->mixed ? collide_batch_prefix<float>(c, 0, B) : collide_batch_prefix<double>(c, 0, B);
    if (s != LP_OK) return s;
    if (which >= 4) LP_TRY(contract<float>(c, Bp, c->q[1]));  // fills the convolution scratch
    auto run = [&]() -> lp_status {
        switch (which) {
        case 0: return c->mixed ? contract<float>(c, Bp, c->q[1]) : contract<double>(c, Bp, c->q[1]);
        case 1:
            if (c->mixed) LP_CUDA(lp::launch_fwd<float>((const float *)c->f, (float2 *)c->t1, (float2 *)c->F, (const float *)c->mfwd, T.n, Bp, c->stream, c->dff));
            else LP_CUDA(lp::launch_fwd<double>((const double *)c->f, (double2 *)c->t1, (double2 *)c->F, (const double *)c->mfwd, T.n, Bp, c->stream));
            return LP_OK;
        case 2:
            LP_CUDA(lp::launch_conserve(c->q[1], c->c1, c->c2, c->cct, T.n3, Bp, c->cpart, c->nchunk, c->lam, c->stream));
            return LP_OK;
        case 3: return c->mixed ? project<float>(c, 0, B, Bp) : project<double>(c, 0, B, Bp);
        default:
            LP_CUDA(lp::launch_computeq_fft((const float2 *)c->F, c->FQC, c->ftw, T.n, Bp, 0, std::min(c->fq_bs, Bp),
                                            c->fscr, c->fq_bs, c->q[1], c->stream, which - 4, nullptr, nullptr,
                                            c->fq_form, c->tc_err));
            return LP_OK;
        }
    };
    LP_TRY(run());
    cudaEvent_t e0, e1;
    LP_CUDA(cudaEventCreate(&e0));
    LP_CUDA(cudaEventCreate(&e1));
    LP_CUDA(cudaEventRecord(e0, c->stream));
    for (int r = 0; r < reps; ++r) LP_TRY(run());
    LP_CUDA(cudaEventRecord(e1, c->stream));
    LP_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    LP_CUDA(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = (double)t / reps;
    return LP_OK;
}

lp_status lp_measure_fp_peaks(double *fp32, double *fp64) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return LP_ERR_NO_DEVICE;
    double *sink = nullptr;
    if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) return LP_ERR_ALLOC;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8;
    double out[2] = {0, 0};
    for (int which = 0; which < 2; ++which) {
        const int iters = which ? 2000 : 20000;
        lp::launch_fma_peak(which == 1, blocks, iters / 10, sink, 0);
        cudaEventRecord(e0, 0);
        lp::launch_fma_peak(which == 1, blocks, iters, sink, 0);
        cudaEventRecord(e1, 0);
        cudaEventSynchronize(e1);
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        // flops: threads * iters * 8 chains * (2 per FMA) * (2 lanes for f32x2)
        const double flops = (double)blocks * 256 * iters * 8 * 2 * (which ? 1 : 2);
        out[which] = t > 0 ? flops / (t * 1e-3) / 1e12 : 0.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (cudaGetLastError() != cudaSuccess) return LP_ERR_CUDA;
    if (fp32) *fp32 = out[0];
    if (fp64) *fp64 = out[1];
    return LP_OK;
}

lp_status lp_moments(lp_ctx *c, double *out) {
    if (!c || !out) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    const lp::Tables &T = c->T;
    const long long kend = (T.prm.fixes & LP_FIX_F3) ? T.size : std::min<long long>(T.size, (long long)T.prm.nx1 * T.nv3);
    LP_CUDA(lp::launch_moments(c->U, T.size, kend, T.nv, T.prm.lv, T.dv, c->mpart, kMomBlocks, c->stream));
    std::vector<double> part(5 * kMomBlocks), px(3 * T.ncell), py(3 * T.ncell);
    LP_CUDA(cudaMemcpyAsync(part.data(), c->mpart, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaMemcpyAsync(px.data(), c->phix, sizeof(double) * px.size(), cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaMemcpyAsync(py.data(), c->phiy, sizeof(double) * py.size(), cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    double s[5] = {0, 0, 0, 0, 0};
    for (int b = 0; b < kMomBlocks; ++b)
        for (int q = 0; q < 5; ++q) s[q] += part[5 * b + q];
    const double dx = T.dx, dy = T.dy, dv = T.dv;
    out[0] = s[0] * dx * dy * T.scalev;
    out[1] = s[1] * dx * dy * dv * dv;
    out[2] = s[2] * dx * dy * dv * dv;
    out[3] = s[3] * dx * dy * dv * dv;
    out[4] = 0.5 * (s[4] * (dx * dy * dv * dv));
    double e = 0.;
    for (int k = 0; k < T.ncell; ++k) {
        e += px[3 * k] * px[3 * k] + py[3 * k] * py[3 * k];
        e += (px[3 * k + 1] * px[3 * k + 1] + py[3 * k + 1] * py[3 * k + 1]) / 12;
        e += (px[3 * k + 2] * px[3 * k + 2] + py[3 * k + 2] * py[3 * k + 2]) / 12;
    }
    out[5] = 0.5 * (dx * dy) * e;
    return LP_OK;
}

}  // extern "C"

// ============================================================== batches
// Many independent runs stepped together.  Runs with equal (n, nv, lv) form
// a class: one collision-only context over the class's concatenated spatial
// cells (its weight table and workspace shared by the runs, per-cell nu and
// dt), whose state buffers hold the runs' states back to back; every run has
// an advection-only context (its own grid, Poisson factors and fields) on
// its slice of those buffers.  A time step advects every run on its own
// stream, then collides every class on its own stream; lp_batch_step
// replays that step from one captured CUDA graph.
struct lp_batch {
    int device = 0;
    cudaStream_t stream = nullptr, own_stream = nullptr;
    std::string err;
    struct Run {
        lp_ctx *adv = nullptr;
        int cls = 0, cell0 = 0;
        cudaStream_t st = nullptr;
        cudaEvent_t done = nullptr;
    };
    struct Cls {
        lp_ctx *eng = nullptr;
        std::vector<int> runs;
        int ncell = 0;
        bool collide = false;  // some run has nu > 0
        double tuned_ms = 0.;
        cudaStream_t st = nullptr;
        cudaEvent_t done = nullptr;
    };
    std::vector<Run> runs;
    std::vector<Cls> cls;
    cudaEvent_t fork = nullptr;
    cudaGraphExec_t gexec = nullptr;
    cudaStream_t gstream = nullptr;
};

namespace {

lp_status bfail(lp_batch *b, lp_status s, const std::string &msg) {
    if (b) b->err = msg;
    return s;
}

#define LPB_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return bfail(b, LP_ERR_CUDA, std::string(#call) + ": " +     \
                                                                cudaGetErrorString(e_));    \
    } while (0)

void batch_destroy(lp_batch *b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (auto &r : b->runs) {
        if (r.adv) { cudaStreamSynchronize(r.adv->stream); destroy(r.adv); }
        if (r.st) cudaStreamDestroy(r.st);
        if (r.done) cudaEventDestroy(r.done);
    }
    for (auto &k : b->cls) {
        if (k.eng) { cudaStreamSynchronize(k.eng->stream); destroy(k.eng); }
        if (k.st) cudaStreamDestroy(k.st);
        if (k.done) cudaEventDestroy(k.done);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
}

// One time step (or one of its halves) of every run, forked from b->stream
// onto the runs' and classes' streams and joined back; also the body of the
// captured step graph.
lp_status batch_body(lp_batch *b, bool adv, bool col) {
    cudaStream_t S = b->stream;
    if (adv) {
        LPB_CUDA(cudaEventRecord(b->fork, S));
        for (auto &r : b->runs) {
            LPB_CUDA(cudaStreamWaitEvent(r.st, b->fork, 0));
            r.adv->stream = r.st;
            const lp_status s = advect(r.adv);
            if (s != LP_OK) return bfail(b, s, "advection: " + r.adv->err);
            LPB_CUDA(cudaEventRecord(r.done, r.st));
            LPB_CUDA(cudaStreamWaitEvent(S, r.done, 0));
        }
    }
    if (col) {
        LPB_CUDA(cudaEventRecord(b->fork, S));
        for (auto &k : b->cls) {
            if (!k.collide) continue;
            LPB_CUDA(cudaStreamWaitEvent(k.st, b->fork, 0));
            k.eng->stream = k.st;
            const lp_status s = collide(k.eng, 0, k.ncell);
            if (s != LP_OK) return bfail(b, s, "collision: " + k.eng->err);
            LPB_CUDA(cudaEventRecord(k.done, k.st));
            LPB_CUDA(cudaStreamWaitEvent(S, k.done, 0));
        }
    }
    return LP_OK;
}

bool batch_ready(lp_batch *b) {
    for (auto &r : b->runs)
        if (!r.adv->has_state) return false;
    return true;
}

// ---- autotuner (shared by contexts and batch classes) ----
// Key of a collision engine's schedule: n, nv, lv, collided cells, precision
// and device name.
std::string engine_key(const lp_ctx *e, int ncell) {
    const lp::Tables &T = e->T;
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, e->device);
    char buf[512];
    snprintf(buf, sizeof(buf), "n%d_nv%d_lv%.17g_cells%d_%s_%s", T.n, T.nv, T.prm.lv, ncell,
             e->mixed ? "mixed" : "fp64", prop.name);
    std::string s(buf);
    for (char &ch : s)
        if (ch == ' ') ch = '-';
    return s;
}

std::vector<std::string> read_tune_cache(const char *path) {
    std::vector<std::string> lines;
    if (path) {
        if (FILE *fp = fopen(path, "r")) {
            char line[768];
            while (fgets(line, sizeof(line), fp)) lines.emplace_back(line);
            fclose(fp);
        }
    }
    return lines;
}

void write_tune_cache(const char *path, const std::vector<std::string> &lines) {
    if (!path) return;
    if (FILE *fp = fopen(path, "w")) {
        for (const auto &l : lines) fputs(l.c_str(), fp);
        fclose(fp);
    }
}

// Applies a cached schedule for `key` to e; returns whether one was found.
// A line is "key cells_per_pass line_warps ms [convolution_form]"; lines
// without the form leave the context's form as it is.
bool tune_lookup(const std::vector<std::string> &lines, const std::string &key, lp_ctx *e, double *ms) {
    bool found = false;
    for (const auto &l : lines) {
        char kbuf[512];
        int bp = 0, lw = 0, form = -1;
        double t = 0.;
        const int nf = sscanf(l.c_str(), "%511s %d %d %lf %d", kbuf, &bp, &lw, &t, &form);
        if (nf >= 4 && key == kbuf && bp >= 32 &&
            bp <= e->Bcap && bp % 32 == 0 && (lw == 2 || lw == 4 || (lw == 0 && e->FQC) || !e->LW)) {
            e->Bpass = bp;
            e->line_warps = e->LW ? lw : 2;
            if (nf == 5 && e->FQC && (form == 0 || form == 1)) e->fq_form = form;
            *ms = t;
            found = true;
        }
    }
    return found;
}

// One collision step of cells [0, ncell) of engine e with its current
// schedule, best of `reps` after a warm-up (CUDA events on st); the state is
// restored from `backup` before every run and only the collision is timed.
lp_status time_engine(lp_ctx *e, int ncell, cudaStream_t st, const double *backup, int reps, double *ms) {
    lp_ctx *c = e;
    const size_t bytes = sizeof(double) * (size_t)e->T.size * 7;
    cudaEvent_t e0, e1;
    LP_CUDA(cudaEventCreate(&e0));
    LP_CUDA(cudaEventCreate(&e1));
    cudaStream_t keep = e->stream;
    e->stream = st;
    double best = 1e300;
    lp_status s = LP_OK;
    for (int i = 0; i <= reps && s == LP_OK; ++i) {
        cudaMemcpyAsync(e->U, backup, bytes, cudaMemcpyDeviceToDevice, st);
        cudaEventRecord(e0, st);
        s = collide(e, 0, ncell);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) s = LP_ERR_CUDA;
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (i > 0) best = std::min(best, (double)t);
    }
    e->stream = keep;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = best;
    return s;
}

// Picks the fastest schedule of engine e for cells [0, ncell): cells per pass
// 64, 128, ... up to the workspace capacity; 2 or 4 warps per line block of
// the line-tiled contraction, or the convolution form in either kernel form
// (axis-2 spectra on chip, or three passes through device memory: the
// first is faster at n <= 24, the second at n = 32).  e->U1 holds the state
// meanwhile.
lp_status tune_engine(lp_ctx *e, int ncell, cudaStream_t st, int reps, double *best_ms) {
    lp_ctx *c = e;
    const size_t bytes = sizeof(double) * (size_t)e->T.size * 7;
    std::vector<int> passes;
    for (int bp = 64; bp < e->Bcap; bp *= 2) passes.push_back(bp);
    passes.push_back(e->Bcap);
    struct Cand {
        int lw, form;
    };
    std::vector<Cand> cands = {{2, e->fq_form}};
    if (e->LW) cands.push_back({4, e->fq_form});
    if (e->FQC) {
        cands.push_back({0, 1});
        cands.push_back({0, 0});
    }
    LP_CUDA(cudaMemcpyAsync(e->U1, e->U, bytes, cudaMemcpyDeviceToDevice, st));
    double best = 1e300;
    int bbp = e->Bcap, blw = 2, bform = e->fq_form;
    for (int bp : passes)
        for (const Cand &cd : cands) {
            e->Bpass = bp;
            e->line_warps = cd.lw;
            e->fq_form = cd.form;
            double ms = 0.;
            LP_TRY(time_engine(e, ncell, st, e->U1, reps, &ms));
            if (ms < best) { best = ms; bbp = bp; blw = cd.lw; bform = cd.form; }
        }
    LP_CUDA(cudaMemcpyAsync(e->U, e->U1, bytes, cudaMemcpyDeviceToDevice, st));
    LP_CUDA(cudaStreamSynchronize(st));
    e->Bpass = bbp;
    e->line_warps = blw;
    e->fq_form = bform;
    *best_ms = best;
    return LP_OK;
}

}  // namespace

extern "C" {

lp_status lp_batch_create(const lp_params *ps, int count, lp_batch **out) {
    if (!ps || !out || count < 1) return LP_ERR_INVALID;
    *out = nullptr;
    const unsigned fixes = ps[0].fixes;
    const int prec = ps[0].precision;
    for (int r = 0; r < count; ++r) {
        if (ps[r].fixes != fixes || ps[r].precision != prec || ps[r].linear_ei != ps[0].linear_ei)
            return LP_ERR_INVALID;  // shared fixes, precision and operator
        const int ncell = ps[r].nx1 * ps[r].nx2;
        const int ncollide = (fixes & LP_FIX_F3) ? ncell : std::min(ps[r].nx1, ncell);
        if (ncollide != ncell) return LP_ERR_INVALID;  // 2-D runs need LP_FIX_F3
    }
    if (!(fixes & LP_FIX_F1)) return LP_ERR_INVALID;  // collisions run in passes of cells
    lp_batch *b = new lp_batch();
    cudaGetDevice(&b->device);
    if (cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
        batch_destroy(b);
        return LP_ERR_CUDA;
    }
    b->stream = b->own_stream;
    // classes by (n, nv, lv), in order of first appearance
    b->runs.resize(count);
    for (int r = 0; r < count; ++r) {
        int k = 0;
        for (; k < (int)b->cls.size(); ++k) {
            const lp_params &q = ps[b->cls[k].runs[0]];
            if (q.n == ps[r].n && q.nv == ps[r].nv && q.lv == ps[r].lv) break;
        }
        if (k == (int)b->cls.size()) b->cls.emplace_back();
        auto &K = b->cls[k];
        b->runs[r].cls = k;
        b->runs[r].cell0 = K.ncell;
        K.runs.push_back(r);
        K.ncell += ps[r].nx1 * ps[r].nx2;
        if (ps[r].nu > 0.) K.collide = true;
    }
    lp_status s = LP_OK;
    for (auto &K : b->cls) {
        lp_params pe = ps[K.runs[0]];
        pe.nx1 = K.ncell; pe.nx2 = 1; pe.nu = 1.0; pe.dt = 1.0;
        CtxOpts o;
        o.advect = false;
        s = ctx_create(&pe, o, &K.eng);
        if (s != LP_OK) break;
        // per-cell nu and dt, padded by one pass
        std::vector<double> nu(K.ncell + K.eng->Bcap, 0.), dt(K.ncell + K.eng->Bcap, 0.);
        for (int r : K.runs) {
            const int nc = ps[r].nx1 * ps[r].nx2;
            for (int i = 0; i < nc; ++i) {
                nu[b->runs[r].cell0 + i] = ps[r].nu;
                dt[b->runs[r].cell0 + i] = ps[r].dt;
            }
        }
        s = upload(K.eng, &K.eng->cnu, nu.data(), nu.size());
        if (s == LP_OK) s = upload(K.eng, &K.eng->cdt, dt.data(), dt.size());
        if (s == LP_OK && (cudaStreamCreateWithFlags(&K.st, cudaStreamNonBlocking) != cudaSuccess ||
                           cudaEventCreateWithFlags(&K.done, cudaEventDisableTiming) != cudaSuccess))
            s = LP_ERR_CUDA;
        if (s != LP_OK) break;
    }
    for (int r = 0; r < count && s == LP_OK; ++r) {
        auto &R = b->runs[r];
        lp_ctx *eng = b->cls[R.cls].eng;
        const size_t off = (size_t)R.cell0 * eng->T.nv3 * 7;
        CtxOpts o;
        o.collide = false;
        o.U = eng->U + off; o.U1 = eng->U1 + off; o.Ut = eng->Ut + off;
        s = ctx_create(&ps[r], o, &R.adv);
        if (s == LP_OK && (cudaStreamCreateWithFlags(&R.st, cudaStreamNonBlocking) != cudaSuccess ||
                           cudaEventCreateWithFlags(&R.done, cudaEventDisableTiming) != cudaSuccess))
            s = LP_ERR_CUDA;
    }
    if (s != LP_OK) {
        batch_destroy(b);
        return s;
    }
    *out = b;
    return LP_OK;
}

lp_status lp_batch_destroy(lp_batch *b) {
    if (!b) return LP_ERR_INVALID;
    batch_destroy(b);
    return LP_OK;
}

lp_status lp_batch_set_stream(lp_batch *b, void *st) {
    if (!b) return LP_ERR_INVALID;
    b->stream = st ? (cudaStream_t)st : b->own_stream;
    return LP_OK;
}

lp_status lp_batch_synchronize(lp_batch *b) {
    if (!b) return LP_ERR_INVALID;
    LPB_CUDA(cudaStreamSynchronize(b->stream));
    return LP_OK;
}

const char *lp_batch_last_error(const lp_batch *b) { return b ? b->err.c_str() : "null batch"; }

size_t lp_batch_device_bytes(const lp_batch *b) {
    if (!b) return 0;
    size_t n = 0;
    for (auto &r : b->runs) n += r.adv->bytes;
    for (auto &k : b->cls) n += k.eng->bytes;
    return n;
}

lp_status lp_batch_set_state(lp_batch *b, int run, const double *U, size_t n) {
    if (!b || run < 0 || run >= (int)b->runs.size()) return LP_ERR_INVALID;
    lp_ctx *c = b->runs[run].adv;
    c->stream = b->stream;
    const lp_status s = lp_set_state(c, U, n);
    return s == LP_OK ? s : bfail(b, s, c->err);
}

lp_status lp_batch_get_state(lp_batch *b, int run, double *U, size_t n) {
    if (!b || run < 0 || run >= (int)b->runs.size()) return LP_ERR_INVALID;
    lp_ctx *c = b->runs[run].adv;
    c->stream = b->stream;
    const lp_status s = lp_get_state(c, U, n);
    return s == LP_OK ? s : bfail(b, s, c->err);
}

lp_status lp_batch_set_init(lp_batch *b, int run, int kind, double u) {
    if (!b || run < 0 || run >= (int)b->runs.size()) return LP_ERR_INVALID;
    lp_ctx *c = b->runs[run].adv;
    c->stream = b->stream;
    const lp_status s = lp_set_init(c, kind, u);
    return s == LP_OK ? s : bfail(b, s, c->err);
}

lp_status lp_batch_moments(lp_batch *b, int run, double *out6) {
    if (!b || run < 0 || run >= (int)b->runs.size()) return LP_ERR_INVALID;
    lp_ctx *c = b->runs[run].adv;
    LPB_CUDA(cudaStreamSynchronize(b->stream));
    c->stream = b->stream;
    const lp_status s = lp_moments(c, out6);
    return s == LP_OK ? s : bfail(b, s, c->err);
}

lp_status lp_batch_advect_step(lp_batch *b) {
    if (!b) return LP_ERR_INVALID;
    if (!batch_ready(b)) return bfail(b, LP_ERR_STATE, "a run has no state");
    return batch_body(b, true, false);
}

lp_status lp_batch_collision_step(lp_batch *b) {
    if (!b) return LP_ERR_INVALID;
    if (!batch_ready(b)) return bfail(b, LP_ERR_STATE, "a run has no state");
    return batch_body(b, false, true);
}

lp_status lp_batch_step(lp_batch *b, int nsteps) {
    NvtxRange r("lp_batch_step");
    if (!b || nsteps < 0) return LP_ERR_INVALID;
    if (!batch_ready(b)) return bfail(b, LP_ERR_STATE, "a run has no state");
    if (nsteps == 0) return LP_OK;
    if (!b->gexec || b->gstream != b->stream) {
        if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
        cudaGraph_t g = nullptr;
        LPB_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const lp_status s = batch_body(b, true, true);
        const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (s != LP_OK) { if (g) cudaGraphDestroy(g); return s; }
        if (e != cudaSuccess) return bfail(b, LP_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
        const cudaError_t e2 = instantiate_step_graph(&b->gexec, g);
        cudaGraphDestroy(g);
        if (e2 != cudaSuccess) return bfail(b, LP_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e2));
        b->gstream = b->stream;
    }
    for (int i = 0; i < nsteps; ++i) LPB_CUDA(cudaGraphLaunch(b->gexec, b->stream));
    return LP_OK;
}

// ---- diagnostics and state I/O ----
lp_status lp_diagnostics(lp_ctx *c, double *out10) {
    if (!c || !out10) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    if (!c->advect_on) return fail(c, LP_ERR_INVALID, "no Poisson tables in this context");
    const lp::Tables &T = c->T;
    LP_TRY(poisson_on(c, c->U));  // pois2d on the state, as before the reference's moment line
    double m[6];
    const lp_status s = lp_moments(c, m);
    if (s != LP_OK) return s;
    const long long kend = (T.prm.fixes & LP_FIX_F3) ? T.size : std::min<long long>(T.size, (long long)T.prm.nx1 * T.nv3);
    LP_CUDA(lp::launch_entropy(c->U, kend, c->mpart, kMomBlocks, c->stream));
    std::vector<double> part(kMomBlocks);
    LP_CUDA(cudaMemcpyAsync(part.data(), c->mpart, sizeof(double) * kMomBlocks, cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    double ent = 0.;
    for (double v : part) ent += v;
    ent *= 0.5 * T.dv * 0.5 * T.dv * 0.5 * T.dv * 0.5 * T.dx;
    const double ee = m[5], r = std::sqrt(ee);
    const double vals[10] = {m[0], m[1], m[2], m[3], m[4], ee, r, std::log(r), m[4] + ee, ent};
    std::memcpy(out10, vals, sizeof(vals));
    return LP_OK;
}

lp_status lp_diagnostics_append(lp_ctx *c, const char *moments_path, const char *entropy_path) {
    if (!c) return LP_ERR_INVALID;
    double d[10];
    const lp_status s = lp_diagnostics(c, d);
    if (s != LP_OK) return s;
    if (moments_path) {
        FILE *fp = fopen(moments_path, "a");
        if (!fp) return fail(c, LP_ERR_INVALID, std::string("cannot open ") + moments_path);
        fprintf(fp, "%11.8g %11.8g %11.8g  %11.8g  %11.8g  %11.8g  %11.8g  %11.8g  %11.8g \n", d[0], d[1], d[2], d[3],
                d[4], d[5], d[6], d[7], d[8]);
        fclose(fp);
    }
    if (entropy_path) {
        FILE *fp = fopen(entropy_path, "a");
        if (!fp) return fail(c, LP_ERR_INVALID, std::string("cannot open ") + entropy_path);
        const double l1 = std::log(std::fabs(d[9]));
        fprintf(fp, "%11.8g %11.8g %11.8g \n", d[9], l1, std::log(std::fabs(l1)));
        fclose(fp);
    }
    return LP_OK;
}

lp_status lp_marginal_x1v1(lp_ctx *c, double *out) {
    if (!c || !out) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    const lp::Tables &T = c->T;
    const size_t n = (size_t)T.prm.nx1 * 4 * T.nv * 4;
    double *d = nullptr;
    LP_CUDA(cudaMallocAsync((void **)&d, sizeof(double) * n, c->stream));
    LP_CUDA(lp::launch_marginal_x1v1(c->U, T.prm.nx1, T.prm.nx2, T.nv, T.dx, T.dv, T.prm.lv, d, c->stream));
    LP_CUDA(cudaMemcpyAsync(out, d, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaFreeAsync(d, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}

lp_status lp_state_append(lp_ctx *c, const char *path) {
    if (!c || !path) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    std::vector<double> U((size_t)c->T.size * 7);
    const lp_status s = lp_get_state(c, U.data(), U.size());
    if (s != LP_OK) return s;
    FILE *fp = fopen(path, "ab");
    if (!fp) return fail(c, LP_ERR_INVALID, std::string("cannot open ") + path);
    const size_t w = fwrite(U.data(), sizeof(double), U.size(), fp);
    fclose(fp);
    return w == U.size() ? LP_OK : fail(c, LP_ERR_INVALID, "short write");
}

lp_status lp_state_restart(lp_ctx *c, const char *path) {
    if (!c || !path) return LP_ERR_INVALID;
    const size_t n = (size_t)c->T.size * 7, bytes = n * sizeof(double);
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(c, LP_ERR_INVALID, std::string("cannot open ") + path);
    fseek(fp, 0, SEEK_END);
    const long len = ftell(fp);
    if (len <= 0 || (size_t)len % bytes != 0) {
        fclose(fp);
        return fail(c, LP_ERR_INVALID, "file size is not a whole number of states");
    }
    std::vector<double> U(n);
    fseek(fp, len - (long)bytes, SEEK_SET);
    const size_t r = fread(U.data(), sizeof(double), n, fp);
    fclose(fp);
    if (r != n) return fail(c, LP_ERR_INVALID, "short read");
    return lp_set_state(c, U.data(), n);
}

// ---- adjoint ----
lp_status lp_set_adjoint_form(lp_ctx *c, int form) {
    if (!c || (form != 0 && form != 1)) return LP_ERR_INVALID;
    c->adj.qvjp_form = form;
    return LP_OK;
}

lp_status lp_field_energy(lp_ctx *c, double *J, double *lamU) {
    if (!c || !J) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    LP_TRY(adj_setup(c));
    LP_TRY(field_energy_at(c, c->U, lamU));
    LP_CUDA(cudaMemcpyAsync(J, c->adj.J, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}

lp_status lp_collision_vjp(lp_ctx *c, const double *lout, double *lin, double *dnu) {
    if (!c || !lout || !lin) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    LP_TRY(adj_setup(c));
    LP_TRY(collide_vjp(c, c->U, lout, lin));
    const lp::Tables &T = c->T;
    std::vector<double> d(std::max(T.ncollide, 1));
    LP_CUDA(cudaMemcpyAsync(d.data(), c->adj.dnu, sizeof(double) * d.size(), cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    if (dnu) {
        *dnu = 0.;
        if (T.prm.nu > 0.)
            for (int i = 0; i < T.ncollide; ++i) *dnu += d[i];
    }
    return LP_OK;
}

lp_status lp_advect_vjp(lp_ctx *c, const double *lout, double *lin) {
    if (!c || !lout || !lin) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    LP_TRY(adj_setup(c));
    auto &A = c->adj;
    const size_t bytes = sizeof(double) * (size_t)c->T.size * 7;
    LP_CUDA(cudaMemcpyAsync(A.Ukeep, c->U, bytes, cudaMemcpyDeviceToDevice, c->stream));
    LP_TRY(advect(c));
    LP_TRY(advect_vjp(c, A.Ukeep, c->U1, c->Ut, lout, lin));
    LP_CUDA(cudaMemcpyAsync(c->U, A.Ukeep, bytes, cudaMemcpyDeviceToDevice, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}

lp_status lp_step_vjp(lp_ctx *c, const double *lout, double *lin, double *dnu) {
    if (!c || !lout || !lin) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    LP_TRY(adj_setup(c));
    auto &A = c->adj;
    const size_t bytes = sizeof(double) * (size_t)c->T.size * 7;
    double dn = 0.;
    LP_CUDA(cudaMemcpyAsync(A.Ukeep, c->U, bytes, cudaMemcpyDeviceToDevice, c->stream));
    LP_CUDA(cudaMemcpyAsync(lin, lout, bytes, cudaMemcpyDeviceToDevice, c->stream));
    LP_TRY(step_vjp(c, A.Ukeep, lin, &dn));
    LP_CUDA(cudaMemcpyAsync(c->U, A.Ukeep, bytes, cudaMemcpyDeviceToDevice, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    if (dnu) *dnu = dn;
    return LP_OK;
}

lp_status lp_field_energy_gradient(lp_ctx *c, int nsteps, int checkpoint, double *J, double *dU0, double *dnu) {
    NvtxRange r("lp_field_energy_gradient (checkpointed adjoint)");
    if (!c || nsteps < 0 || checkpoint < 1 || !J || !dU0) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    LP_TRY(adj_setup(c));
    auto &A = c->adj;
    const lp::Tables &T = c->T;
    const size_t rec = (size_t)T.size * 7, bytes = sizeof(double) * rec;
    // checkpoints every `checkpoint` steps (index 0: the initial state)
    const int nck = (nsteps + checkpoint - 1) / checkpoint + 1;
    while ((int)A.ck.size() < nck) {
        double *p = nullptr;
        LP_TRY(dalloc(c, &p, rec));
        A.ck.push_back(p);
    }
    if (A.seg_len < checkpoint) {
        LP_TRY(dalloc(c, &A.seg, rec * (size_t)checkpoint));
        A.seg_len = checkpoint;
    }
    LP_CUDA(cudaMemcpyAsync(A.ck[0], c->U, bytes, cudaMemcpyDeviceToDevice, c->stream));
    for (int s = 0; s < nsteps; ++s) {
        if (s > 0 && s % checkpoint == 0)
            LP_CUDA(cudaMemcpyAsync(A.ck[s / checkpoint], c->U, bytes, cudaMemcpyDeviceToDevice, c->stream));
        LP_TRY(one_step(c));
    }
    // J and dJ/dU at the final state
    LP_CUDA(cudaMemcpyAsync(A.Ukeep, c->U, bytes, cudaMemcpyDeviceToDevice, c->stream));
    LP_TRY(field_energy_at(c, A.Ukeep, dU0));
    LP_CUDA(cudaMemcpyAsync(J, A.J, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    double dn = 0.;
    for (int seg = (nsteps - 1) / checkpoint; seg >= 0 && nsteps > 0; --seg) {
        const int s0 = seg * checkpoint, s1 = std::min(nsteps, s0 + checkpoint);
        // recompute the segment's states from its checkpoint
        LP_CUDA(cudaMemcpyAsync(c->U, A.ck[seg], bytes, cudaMemcpyDeviceToDevice, c->stream));
        for (int s = s0; s < s1; ++s) {
            LP_CUDA(cudaMemcpyAsync(A.seg + rec * (size_t)(s - s0), c->U, bytes, cudaMemcpyDeviceToDevice, c->stream));
            if (s + 1 < s1) LP_TRY(one_step(c));
        }
        for (int s = s1 - 1; s >= s0; --s) LP_TRY(step_vjp(c, A.seg + rec * (size_t)(s - s0), dU0, &dn));
    }
    // the context's state is the initial state again
    LP_CUDA(cudaMemcpyAsync(c->U, A.ck[0], bytes, cudaMemcpyDeviceToDevice, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    if (dnu) *dnu = dn;
    return LP_OK;
}

int lp_batch_classes(const lp_batch *b) { return b ? (int)b->cls.size() : 0; }

lp_status lp_batch_class_info(const lp_batch *b, int k, int *info6, double *tuned_ms) {
    if (!b || k < 0 || k >= (int)b->cls.size() || !info6) return LP_ERR_INVALID;
    const auto &K = b->cls[k];
    info6[0] = K.eng->T.n; info6[1] = K.eng->T.nv; info6[2] = (int)K.runs.size(); info6[3] = K.ncell;
    info6[4] = K.eng->Bpass; info6[5] = K.eng->line_warps;
    if (tuned_ms) *tuned_ms = K.tuned_ms;
    return LP_OK;
}

lp_status lp_batch_autotune(lp_batch *b, int reps, const char *cache_path) {
    if (!b || reps < 1) return LP_ERR_INVALID;
    if (!batch_ready(b)) return bfail(b, LP_ERR_STATE, "a run has no state");
    LPB_CUDA(cudaStreamSynchronize(b->stream));
    std::vector<std::string> lines = read_tune_cache(cache_path);  // "key pass_cells line_warps ms"
    bool changed = false;
    for (auto &K : b->cls) {
        const std::string key = engine_key(K.eng, K.ncell);
        if (tune_lookup(lines, key, K.eng, &K.tuned_ms) || !K.collide) continue;
        const lp_status s = tune_engine(K.eng, K.ncell, b->stream, reps, &K.tuned_ms);
        if (s != LP_OK) return bfail(b, s, "autotune: " + K.eng->err);
        char line[768];
        snprintf(line, sizeof(line), "%s %d %d %.6f %d\n", key.c_str(), K.eng->Bpass, K.eng->line_warps, K.tuned_ms,
                 K.eng->fq_form);
        lines.emplace_back(line);
        changed = true;
    }
    if (changed) write_tune_cache(cache_path, lines);
    if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }  // recapture with the new schedule
    return LP_OK;
}

lp_status lp_autotune(lp_ctx *c, int reps, const char *cache_path, int *pass_cells, int *line_warps) {
    if (!c || reps < 1) return LP_ERR_INVALID;
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    if (!c->collide_on) return fail(c, LP_ERR_INVALID, "no collision tables in this context");
    LP_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<std::string> lines = read_tune_cache(cache_path);
    const std::string key = engine_key(c, c->T.ncollide);
    double ms = 0.;
    if (!tune_lookup(lines, key, c, &ms) && c->T.ncollide > 0) {
        LP_TRY(tune_engine(c, c->T.ncollide, c->stream, reps, &ms));
        char line[768];
        snprintf(line, sizeof(line), "%s %d %d %.6f %d\n", key.c_str(), c->Bpass, c->line_warps, ms, c->fq_form);
        lines.emplace_back(line);
        write_tune_cache(cache_path, lines);
    }
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }  // recapture with the new schedule
    if (c->cgexec) { cudaGraphExecDestroy(c->cgexec); c->cgexec = nullptr; }
    if (pass_cells) *pass_cells = c->Bpass;
    if (line_warps) *line_warps = c->line_warps;
    return LP_OK;
}

lp_status lp_set_convolution_form(lp_ctx *c, int form) {
    if (!c) return LP_ERR_INVALID;
    if (form != 0 && form != 1) return fail(c, LP_ERR_INVALID, "convolution form must be 0 or 1");
    if (!c->FQC) return fail(c, LP_ERR_INVALID, "no convolution form in this context");
    LP_CUDA(cudaStreamSynchronize(c->stream));
    c->fq_form = form;
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }  // recapture with the new kernels
    if (c->cgexec) { cudaGraphExecDestroy(c->cgexec); c->cgexec = nullptr; }
    return LP_OK;
}

lp_status lp_get_convolution_form(const lp_ctx *c, int *form) {
    if (!c || !form) return LP_ERR_INVALID;
    *form = c->FQC ? c->fq_form : -1;
    return LP_OK;
}

lp_status lp_set_schedule(lp_ctx *c, int pass_cells, int line_warps) {
    if (!c) return LP_ERR_INVALID;
    if (!c->collide_on) return fail(c, LP_ERR_INVALID, "no collision tables in this context");
    if (pass_cells < 32 || pass_cells % 32 || pass_cells > c->Bcap)
        return fail(c, LP_ERR_INVALID, "pass_cells must be a multiple of 32 up to the workspace capacity");
    const bool ok = (line_warps == 2) || (line_warps == 4 && c->LW) || (line_warps == 0 && c->FQC);
    if (!ok) return fail(c, LP_ERR_INVALID, "contraction form not available in this context");
    LP_CUDA(cudaStreamSynchronize(c->stream));
    c->Bpass = pass_cells;
    c->line_warps = line_warps;
    if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
    if (c->cgexec) { cudaGraphExecDestroy(c->cgexec); c->cgexec = nullptr; }
    return LP_OK;
}

}  // extern "C"

// ============================================================== x1 slabs
// A sharded run splits the x1 rows of the spatial grid into contiguous slabs,
// one per rank (the reference splits the cells over MPI ranks at
// LP_ompi_1.cpp:164-178 and re-assembles the whole state on every rank with a
// root gather and broadcast, LP_ompi_1.cpp:518-567, advection_1.cpp:472-489).
// Here a rank keeps only its slab plus one halo row on each side:
//   - collisions are local to a spatial cell: no exchange;
//   - each SSP-RK3 stage needs the neighbours' edge rows (the x1 upwind flux
//     of I3 reads one row to each side) -- the caller exchanges them into the
//     halo rows of the stage buffer;
//   - each stage needs the field of the whole grid: the caller all-gathers
//     the three charge moments of every cell, and every rank solves the same
//     (small) LDG Poisson system redundantly.
// The exchanges themselves are the caller's (torch.distributed in the
// package's slab schedule); these entry points do the device work.

namespace {

// Field integrals of the slab's local rows (halo rows included, periodic in
// x1) from those of the whole grid; layout [14][cells] on both sides.
__global__ void k_slab_fields(const double *__restrict__ gf, int gnc, double *__restrict__ f, int nc, int nx2,
                              int i1_off, int gnx1) {
    lp::lp_grid_wait();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nc) return;
    const int i1 = s / nx2, i2 = s % nx2;
    int g = (i1 + i1_off) % gnx1;
    if (g < 0) g += gnx1;
    const int gs = g * nx2 + i2;
#pragma unroll
    for (int q = 0; q < 14; ++q) f[q * nc + s] = gf[q * gnc + gs];
}

double *stage_buffer(lp_ctx *c, int stage) { return stage == 0 ? c->U : stage == 1 ? c->U1 : c->Ut; }

}  // namespace

extern "C" {

lp_status lp_slab_create(const lp_params *g, int i1_begin, int i1_end, lp_ctx **out) {
    if (!g || !out) return LP_ERR_INVALID;
    *out = nullptr;
    if (g->nx1 < 2 || g->nx2 < 1 || i1_begin < 0 || i1_end > g->nx1 || i1_end - i1_begin < 1)
        return LP_ERR_INVALID;
    lp::Tables gt;
    std::string err;
    lp_status s = lp::build_tables(*g, gt, err, lp::kTablesPoisson);
    if (s != LP_OK) return s;
    lp_params p = *g;
    p.nx1 = i1_end - i1_begin + 2;
    lp_ctx *c = nullptr;
    s = ctx_create(&p, CtxOpts{}, &c);
    if (s != LP_OK) return s;
    // the global cell sizes (the local geometry's lx / nx1 can differ in the
    // last bit), the slab's place in the global grid, the global Poisson factors
    c->T.dx = gt.dx;
    c->T.dy = gt.dy;
    c->i1_off = i1_begin - 1;
    c->slab_gnx1 = g->nx1;
    c->slab_nown = i1_end - i1_begin;
    c->gpois = gt.pois;
    const size_t gnc = (size_t)g->nx1 * g->nx2;
    s = upload(c, &c->gab, gt.pois.ab.data(), gt.pois.ab.size());
    if (s == LP_OK) s = upload(c, &c->gipiv, gt.pois.ipiv.data(), gt.pois.ipiv.size());
    if (s == LP_OK) s = upload(c, &c->ggate, gt.pois.gate.data(), gt.pois.gate.size());
    if (s == LP_OK) s = dalloc(c, &c->gpb, (size_t)gt.pois.ndim);
    if (s == LP_OK) s = dalloc(c, &c->gpotc, 3 * gnc);
    if (s == LP_OK) s = dalloc(c, &c->gphix, 3 * gnc);
    if (s == LP_OK) s = dalloc(c, &c->gphiy, 3 * gnc);
    if (s == LP_OK) s = dalloc(c, &c->gfields, 14 * gnc);
    if (s == LP_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) s = LP_ERR_CUDA;
    if (s != LP_OK) {
        destroy(c);
        return s;
    }
    *out = c;
    return LP_OK;
}

lp_status lp_stage_device_ptr(lp_ctx *c, int stage, double **dev) {
    if (!c || !dev || stage < 0 || stage > 2) return LP_ERR_INVALID;
    *dev = stage_buffer(c, stage);
    if (stage == 0) c->has_state = true;
    return LP_OK;
}

lp_status lp_slab_charge(lp_ctx *c, int stage, double *rt_dev) {
    if (!c || !rt_dev || stage < 0 || stage > 2) return LP_ERR_INVALID;
    if (!c->slab_gnx1) return fail(c, LP_ERR_INVALID, "not a slab context");
    const int nx2 = c->T.prm.nx2;
    const double *Us = stage_buffer(c, stage) + (size_t)nx2 * c->T.nv3 * 7;  // skip halo row 0
    LP_CUDA(lp::launch_charge(Us, c->slab_nown * nx2, c->T.nv3, c->T.scalev, rt_dev, c->stream));
    return LP_OK;
}

lp_status lp_slab_fields(lp_ctx *c, const double *rt_global_dev) {
    if (!c || !rt_global_dev) return LP_ERR_INVALID;
    if (!c->slab_gnx1) return fail(c, LP_ERR_INVALID, "not a slab context");
    const int nx2 = c->T.prm.nx2, gnc = c->slab_gnx1 * nx2;
    LP_CUDA(lp::launch_poisson(poisson_dev_of(c->gpois, c->gab, c->gipiv, c->ggate), rt_global_dev, 1, c->gpb,
                               c->gpotc, c->gphix, c->gphiy, c->gfields, c->stream));
    k_slab_fields<<<(c->T.ncell + 127) / 128, 128, 0, c->stream>>>(c->gfields, gnc, c->fields, c->T.ncell, nx2,
                                                                   c->i1_off, c->slab_gnx1);
    LP_CUDA(cudaGetLastError());
    return LP_OK;
}

lp_status lp_slab_advect_stage(lp_ctx *c, int stage) {
    if (!c || stage < 0 || stage > 2) return LP_ERR_INVALID;
    if (!c->slab_gnx1) return fail(c, LP_ERR_INVALID, "not a slab context");
    if (!c->has_state) return fail(c, LP_ERR_STATE, "no state uploaded");
    double *out = stage == 0 ? c->U1 : stage == 1 ? c->Ut : c->U;
    LP_CUDA(lp::launch_flux_stage(advect_dev(c), c->U, stage_buffer(c, stage), nullptr, c->fields, stage, out,
                                  nullptr, nullptr, c->stream));
    return LP_OK;
}

lp_status lp_slab_fields_host(lp_ctx *c, double *potc, double *phix, double *phiy) {
    if (!c) return LP_ERR_INVALID;
    if (!c->slab_gnx1) return fail(c, LP_ERR_INVALID, "not a slab context");
    const size_t n = 3 * (size_t)c->slab_gnx1 * c->T.prm.nx2;
    if (potc) LP_CUDA(cudaMemcpyAsync(potc, c->gpotc, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (phix) LP_CUDA(cudaMemcpyAsync(phix, c->gphix, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (phiy) LP_CUDA(cudaMemcpyAsync(phiy, c->gphiy, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    LP_CUDA(cudaStreamSynchronize(c->stream));
    return LP_OK;
}

}  // extern "C"
