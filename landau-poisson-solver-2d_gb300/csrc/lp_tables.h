// Host-side tables of the GB300 Landau-Poisson hot path: grids, the
// omega-dependent factors of the Landau weight, the conservation rows and
// their inverse Gram matrix, the per-axis DG projection factors, the
// phase-folded per-axis DFT matrices and the factored LDG Poisson band
// matrix.  Computed once per context in FP64 on the host (compiled with
// -ffp-contract=off: several closed forms of the reference are evaluated in
// the same operation order so that ill-conditioned cases give the same
// values), then uploaded.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "lp_gb300.h"

namespace lp {

struct PoissonTables {
    int nx = 0, ny = 0, ndim = 0, kl = 0, ku = 0, ldab = 0;
    std::vector<double> ab;   // LU factors in LAPACK band storage, ldab x ndim
    std::vector<int> ipiv;    // 1-based pivots
    double dxp = 0, dyp = 0;
    // 3x3 post-processing blocks (row-major [k][kk])
    double acvx[9], acyrr[9], acyrl[9], acvy[9], acxrr[9], acxrl[9];
    std::vector<uint8_t> gate;  // per x1 cell: centre coincides with the top gate
};

struct Tables {
    lp_params prm{};
    int n = 0, nv = 0, n3 = 0, nv3 = 0, ncell = 0;
    long long size = 0;  // records
    double PI = 0, L_v = 0, R_v = 0, L_eta = 0, h_eta = 0, h_v = 0, dv = 0, dx = 0, dy = 0;
    double scale = 0, scale3 = 0, scaleL = 0, scalev = 0;
    std::vector<double> v, eta, wt;
    std::vector<double> shat;    // n3 x 6: Shat00, 01, 02, 11, 12, 22
    std::vector<double> ahat;    // n3
    std::vector<uint8_t> rzero;  // n3
    std::vector<double> cw;      // n3: h_eta^3 wt_l wt_m wt_n (reference factor order)
    std::vector<double> c1, c2;  // 5 x n3
    double cct_inv[25] = {0};
    std::vector<int> nodecell;   // n
    std::vector<double> nodeoff; // n: (v[l] - Gridv(nodecell[l])) / dv
    std::vector<double> tfac;    // 3 x n x nv complex (T0, T1, T2)
    std::vector<double> mfwd;    // n x n complex, out index major
    std::vector<double> minv;    // n x n complex, out index major
    // The same two matrices factored as M[a][i] = post[a] w^((a i) mod n) pre[i],
    // w = exp(-2 pi i / n) for the forward ([0]) and its conjugate for the
    // inverse ([1]): n complex entries each.  dft_fac_ok: the factors give
    // the matrices back to 1e-12 of their largest entry.
    std::vector<double> dpre[2], dpost[2], dw[2];
    bool dft_fac_ok = false;
    std::vector<int> pair_off;   // n3 + 1 prefix offsets of the pair table
    // two-species variant: n3 + 1 prefix offsets of the window entries (the
    // linear weight table) and CCt_linear's inverse embedded in rows/columns
    // {0, 4} of a 5x5 matrix (zero elsewhere)
    std::vector<long long> win_off;
    double cct_lin5[25] = {0};
    // Moment reconciliation of the mixed path: the 5 DG moments (mass, three
    // momenta, kinetic energy) of a cell's collision increment equal
    // dt*kfac*Re sum_k gmom[m][k] Qc(k) exactly; gm_inv is the inverse of
    // sum_j Phi_j Phi_j^T over the velocity cells of one spatial cell.
    std::vector<double> gmom;    // 5 x n3 complex
    double gm_inv[25] = {0};
    PoissonTables pois;
    int ncollide = 0;            // spatial cells that are collided
};

// Validates p and fills t (grids and constants always, the collision and the
// Poisson tables as `parts` asks); returns LP_OK or LP_ERR_INVALID with err set.
constexpr unsigned kTablesCollision = 1u, kTablesPoisson = 2u, kTablesAll = 3u;
lp_status build_tables(const lp_params &p, Tables &t, std::string &err, unsigned parts = kTablesAll);

// Dense inverse of the LDG Poisson matrix (row-major ndim x ndim) from the
// band LU factors.
void poisson_inverse(const PoissonTables &ps, std::vector<double> &inv);

// gHat3(eta_xi, eta_omega) from the omega tables (the reference's order).
double weight_host(const Tables &t, int xi, int om);

}  // namespace lp
