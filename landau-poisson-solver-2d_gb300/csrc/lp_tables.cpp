// Host-side table construction for the GB300 Landau-Poisson hot path.
// Citations are to the reference checkout:
//   C = source/collisionRoutines_1.cpp   K = source/conservationRoutines.cpp
//   P = source/PoissonFunctions.cpp      M = source/LP_ompi_1.cpp
//   S = source/SetInit_1.cpp             A = source/advection_1.cpp
#include "lp_tables.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace lp {
namespace {

// ---- Landau weight, omega part (C:10-28, C:47-53, C:67) -------------------
struct WeightFns {
    double PI, R;
    double s1(double k1, double k2, double k3) const {
        if (k1 == 0. && k2 == 0. && k3 == 0.) return std::sqrt(1. / (2 * PI)) * R * R;
        return std::sqrt(2.0 / PI) * (1 - std::cos(R * std::sqrt(k1 * k1 + k2 * k2 + k3 * k3))) /
               (k1 * k1 + k2 * k2 + k3 * k3);
    }
    double s233(double k1, double k2, double k3) const {
        double r = std::sqrt(k1 * k1 + k2 * k2 + k3 * k3);
        if (r == 0.) return std::sqrt(1. / (2. * PI)) * R * R / 3.;
        return std::sqrt(2. / PI) *
               ((k1 * k1 + k2 * k2) * (R * r - std::sin(R * r)) / (R * r) -
                k3 * k3 * (R * r + R * r * std::cos(R * r) - 2. * std::sin(R * r)) / (R * r)) /
               std::pow(r, 4.);
    }
    double s213(double k1, double k2, double k3) const {
        double r = std::sqrt(k1 * k1 + k2 * k2 + k3 * k3);
        if (k1 == 0. || k3 == 0.) return 0.;
        return -std::sqrt(2 / PI) * k1 * k3 * (2. * R * r + R * r * std::cos(R * r) - 3. * std::sin(R * r)) /
               (R * std::pow(r, 5.));
    }
};

double sinc(double x) { return x == 0.0 ? 1.0 : std::sin(x) / x; }

// ---- LAPACK restatements (unblocked DGETF2/DGETRI, DGBTF2) ----------------
int dgetf2(int m, int n, double *a, int lda, int *ipiv) {
    auto A = [&](int i, int j) -> double & { return a[(i - 1) + (long)(j - 1) * lda]; };
    int info = 0;
    for (int j = 1; j <= std::min(m, n); ++j) {
        int jp = j;
        double amax = std::fabs(A(j, j));
        for (int i = j + 1; i <= m; ++i)
            if (std::fabs(A(i, j)) > amax) { amax = std::fabs(A(i, j)); jp = i; }
        ipiv[j - 1] = jp;
        if (A(jp, j) != 0.0) {
            if (jp != j)
                for (int c = 1; c <= n; ++c) std::swap(A(j, c), A(jp, c));
            if (j < m) {
                double r = 1.0 / A(j, j);
                for (int i = j + 1; i <= m; ++i) A(i, j) *= r;
            }
        } else if (info == 0) {
            info = j;
        }
        if (j < std::min(m, n))
            for (int c = j + 1; c <= n; ++c) {
                double y = A(j, c);
                if (y != 0.0) {
                    double t = -y;
                    for (int i = j + 1; i <= m; ++i) A(i, c) += A(i, j) * t;
                }
            }
    }
    return info;
}

int dgetri(int n, double *a, int lda, const int *ipiv) {
    auto A = [&](int i, int j) -> double & { return a[(i - 1) + (long)(j - 1) * lda]; };
    std::vector<double> work(n);
    for (int j = 1; j <= n; ++j)
        if (A(j, j) == 0.0) return j;
    for (int j = 1; j <= n; ++j) {
        A(j, j) = 1.0 / A(j, j);
        double ajj = -A(j, j);
        for (int jj = 1; jj <= j - 1; ++jj) {
            double xj = A(jj, j);
            if (xj != 0.0) {
                for (int i = 1; i <= jj - 1; ++i) A(i, j) += xj * A(i, jj);
                A(jj, j) = A(jj, j) * A(jj, jj);
            }
        }
        for (int i = 1; i <= j - 1; ++i) A(i, j) *= ajj;
    }
    for (int j = n; j >= 1; --j) {
        for (int i = j + 1; i <= n; ++i) { work[i - 1] = A(i, j); A(i, j) = 0.0; }
        if (j < n)
            for (int jj = j + 1; jj <= n; ++jj) {
                double t = -work[jj - 1];
                if (work[jj - 1] != 0.0)
                    for (int i = 1; i <= n; ++i) A(i, j) += t * A(i, jj);
            }
    }
    for (int j = n - 1; j >= 1; --j) {
        int jp = ipiv[j - 1];
        if (jp != j)
            for (int i = 1; i <= n; ++i) std::swap(A(i, j), A(i, jp));
    }
    return 0;
}

int dgbtf2(int m, int n, int kl, int ku, double *ab, int ldab, int *ipiv) {
    auto AB = [&](int i, int j) -> double & { return ab[(i - 1) + (long)(j - 1) * ldab]; };
    int info = 0, kv = ku + kl;
    for (int j = ku + 2; j <= std::min(kv, n); ++j)
        for (int i = kv - j + 2; i <= kl; ++i) AB(i, j) = 0.0;
    int ju = 1;
    for (int j = 1; j <= std::min(m, n); ++j) {
        if (j + kv <= n)
            for (int i = 1; i <= kl; ++i) AB(i, j + kv) = 0.0;
        int km = std::min(kl, m - j);
        int jp = 1;
        double amax = std::fabs(AB(kv + 1, j));
        for (int i = 2; i <= km + 1; ++i)
            if (std::fabs(AB(kv + i, j)) > amax) { amax = std::fabs(AB(kv + i, j)); jp = i; }
        ipiv[j - 1] = jp + j - 1;
        if (AB(kv + jp, j) != 0.0) {
            ju = std::max(ju, std::min(j + ku + jp - 1, n));
            if (jp != 1)
                for (int c = 0; c <= ju - j; ++c) std::swap(AB(kv + jp - c, j + c), AB(kv + 1 - c, j + c));
            if (km > 0) {
                double r = 1.0 / AB(kv + 1, j);
                for (int i = 1; i <= km; ++i) AB(kv + 1 + i, j) *= r;
                for (int c = 1; c <= ju - j; ++c) {
                    double y = AB(kv - c + 1, j + c);
                    if (y != 0.0) {
                        double t = -y;
                        for (int i = 1; i <= km; ++i) AB(kv + i - c + 1, j + c) += AB(kv + 1 + i, j) * t;
                    }
                }
            }
        } else if (info == 0) {
            info = j;
        }
    }
    return info;
}

// ---- LDG Poisson assembly --------------------------
double fle(int k, double x) { return k == 0 ? 1.0 : (k == 1 ? x : x * x - 1. / 12.); }
double fled(int k, double x) { return k == 0 ? 0. : (k == 1 ? 1. : 2. * x); }

lp_status build_poisson(Tables &t, std::string &err) {
    PoissonTables &ps = t.pois;
    const int NX = t.prm.nx1, NY = t.prm.nx2;
    ps.nx = NX; ps.ny = NY;
    const double xlength = t.prm.lx, ylength = t.prm.lx;
    std::vector<double> DX(NX + 2, 0.), DY(NY + 2, 0.), CX(NX + 2, 0.);
    for (int i = 1; i <= NX; ++i) DX[i] = xlength / ((double)NX);
    for (int j = 1; j <= NY; ++j) DY[j] = ylength / ((double)NY);
    CX[1] = 0. + DX[1] / 2.;
    for (int i = 2; i <= NX; ++i) CX[i] = CX[i - 1] + DX[i - 1] / 2. + DX[i] / 2.;
    const double xa = CX[1] - DX[1] / 2., xb = CX[NX] + DX[NX] / 2.;
    const double xc = xa + (xb - xa) / 2., xd = xa + (xb - xa) / 2.;
    ps.dxp = DX[1]; ps.dyp = DY[1];
    ps.gate.assign(NX + 2, 0);
    for (int ix = 1; ix <= NX; ++ix) ps.gate[ix] = (CX[ix] >= xc && CX[ix] <= xd);

    const double s3 = std::sqrt(3.0) / 6.0;
    const double gp[3] = {0., -s3, s3}, gw[3] = {0., 0.5, 0.5};
    double gaut[3][3];
    for (int l = 1; l <= 2; ++l)
        for (int ll = 1; ll <= 2; ++ll) gaut[l][ll] = gw[l] * gw[ll];
    const double ai[3] = {1., 12.0, 12.0};
    static const int DXG[3] = {0, 1, 0}, DYG[3] = {0, 0, 1};  // modes: 1, x, y
    double bl[3][3], br[3][3], bb[3][3], bt[3][3], cxv[3][3][3], cyv[3][3][3], cxy[3][3][3];
    for (int l = 1; l <= 2; ++l)
        for (int md = 0; md < 3; ++md) {
            bl[md][l] = fle(DXG[md], -0.5) * fle(DYG[md], gp[l]);
            br[md][l] = fle(DXG[md], 0.5) * fle(DYG[md], gp[l]);
            bb[md][l] = fle(DYG[md], -0.5) * fle(DXG[md], gp[l]);
            bt[md][l] = fle(DYG[md], 0.5) * fle(DXG[md], gp[l]);
        }
    for (int l = 1; l <= 2; ++l)
        for (int ll = 1; ll <= 2; ++ll)
            for (int md = 0; md < 3; ++md) {
                cxv[md][l][ll] = fled(DXG[md], gp[l]) * fle(DYG[md], gp[ll]);
                cyv[md][l][ll] = fle(DXG[md], gp[l]) * fled(DYG[md], gp[ll]);
                cxy[md][l][ll] = fle(DXG[md], gp[l]) * fle(DYG[md], gp[ll]);
            }
    double cvx[3][3], cvy[3][3], cyll[3][3], cylr[3][3], cyrl[3][3], cyrr[3][3], cxll[3][3], cxlr[3][3],
        cxrl[3][3], cxrr[3][3];
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
            cvx[i][j] = 0.; cvy[i][j] = 0.;
            for (int kx = 1; kx <= 2; ++kx)
                for (int ky = 1; ky <= 2; ++ky) {
                    cvx[i][j] = cvx[i][j] - cxy[j][kx][ky] * cxv[i][kx][ky] * gaut[kx][ky];
                    cvy[i][j] = cvy[i][j] - cxy[j][kx][ky] * cyv[i][kx][ky] * gaut[kx][ky];
                }
            cyll[i][j] = cylr[i][j] = cyrl[i][j] = cyrr[i][j] = 0.;
            cxll[i][j] = cxlr[i][j] = cxrl[i][j] = cxrr[i][j] = 0.;
        }
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i)
            for (int g = 1; g <= 2; ++g) {
                cyll[i][j] = cyll[i][j] + bl[i][g] * bl[j][g] * gw[g];
                cylr[i][j] = cylr[i][j] + br[i][g] * bl[j][g] * gw[g];
                cyrl[i][j] = cyrl[i][j] + bl[i][g] * br[j][g] * gw[g];
                cyrr[i][j] = cyrr[i][j] + br[i][g] * br[j][g] * gw[g];
                cxll[i][j] = cxll[i][j] + bb[i][g] * bb[j][g] * gw[g];
                cxlr[i][j] = cxlr[i][j] + bt[i][g] * bb[j][g] * gw[g];
                cxrl[i][j] = cxrl[i][j] + bb[i][g] * bt[j][g] * gw[g];
                cxrr[i][j] = cxrr[i][j] + bt[i][g] * bt[j][g] * gw[g];
            }
    double acvx[3][3], acvy[3][3], acyrl[3][3], acyrr[3][3], acxll[3][3], acxrl[3][3], acxrr[3][3];
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
            acvx[i][j] = ai[i] * cvx[i][j]; acvy[i][j] = ai[i] * cvy[i][j];
            acyrl[i][j] = ai[i] * cyrl[i][j]; acyrr[i][j] = ai[i] * cyrr[i][j];
            acxll[i][j] = ai[i] * cxll[i][j]; acxrr[i][j] = ai[i] * cxrr[i][j];
            acxrl[i][j] = ai[i] * cxrl[i][j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            ps.acvx[3 * i + j] = acvx[i][j]; ps.acyrr[3 * i + j] = acyrr[i][j];
            ps.acyrl[3 * i + j] = acyrl[i][j]; ps.acvy[3 * i + j] = acvy[i][j];
            ps.acxrr[3 * i + j] = acxrr[i][j]; ps.acxrl[3 * i + j] = acxrl[i][j];
        }

    const double c11 = 1.;
    const int nsub = (NY + 1) * 3 - 1, nsuper = nsub;
    const int ldab = 2 * nsub + nsuper + 1, m1 = nsub + nsuper + 1;
    const int ndim = 3 * NX * NY;
    ps.kl = nsub; ps.ku = nsuper; ps.ldab = ldab; ps.ndim = ndim;
    ps.ab.assign((size_t)ldab * ndim, 0.);
    ps.ipiv.assign(ndim, 0);
    auto ABP = [&](int r, int col) -> double & { return ps.ab[(r - 1) + (size_t)(col - 1) * ldab]; };
    for (int ix = 1; ix <= NX; ++ix)
        for (int jy = 1; jy <= NY; ++jy) {
            const int ii = (ix - 1) * NY + jy;
            const bool top = (jy == NY), right = (ix == NX), gate = ps.gate[ix] != 0;
            const double ep = 1., epr = right ? 0. : 1., ept = top ? 0. : 1.;
            const double dxr = DX[ix + 1], dyt = DY[jy + 1];
            double col[3][3], cob[3][3], coc[3][3], cott[3][3], cor[3][3];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double vcol = 0., vcob = 0., vcoc = 0., vcott = 0., vcor = 0.;
                    for (int k = 0; k < 3; ++k) {
                        vcol = vcol - (cvx[i][k] - cyll[i][k]) * ep * acyrl[k][j] * DY[jy] / DX[ix];
                        vcob = vcob - (cvy[i][k] - cxll[i][k]) * ep * acxrl[k][j] * DX[ix] / DY[jy];
                        if (!top) vcott = vcott + cxlr[i][k] * ept * (acvy[k][j] + acxrr[k][j]) * DX[ix] / dyt;
                        if (!right) vcor = vcor + cylr[i][k] * (acvx[k][j] + acyrr[k][j]) * epr * DY[jy] / dxr;
                        if (!top && !right)
                            vcoc = vcoc + (cvx[i][k] - cyll[i][k]) * ep * (acvx[k][j] + acyrr[k][j]) * DY[jy] / DX[ix] +
                                   (cvy[i][k] - cxll[i][k]) * ep * (acvy[k][j] + acxrr[k][j]) * DX[ix] / DY[jy] -
                                   cylr[i][k] * acyrl[k][j] * epr * DY[jy] / dxr -
                                   cxlr[i][k] * acxrl[k][j] * ept * DX[ix] / dyt;
                    }
                    vcol = vcol - c11 * cyrl[i][j] * DY[jy];
                    vcob = vcob - c11 * cxrl[i][j] * DX[ix];
                    vcoc = vcoc + c11 * (cyrr[i][j] + cyll[i][j]) * DY[jy] + c11 * (cxrr[i][j] + cxll[i][j]) * DX[ix];
                    vcott = vcott - c11 * cxlr[i][j] * DX[ix];
                    vcor = vcor - c11 * cylr[i][j] * DY[jy];
                    if (top && !right && !gate) {  // Neumann top
                        vcoc = 0.;
                        for (int k = 0; k < 3; ++k)
                            vcoc = vcoc + (cvx[i][k] - cyll[i][k]) * ep * (acvx[k][j] + acyrr[k][j]) * DY[jy] / DX[ix] +
                                   (cvy[i][k] - cxll[i][k]) * ep * (acvy[k][j] + acxrr[k][j]) * DX[ix] / DY[jy] -
                                   cylr[i][k] * acyrl[k][j] * epr * DY[jy] / dxr;
                        vcoc = vcoc + c11 * (cyrr[i][j] + cyll[i][j]) * DY[jy] + c11 * cxll[i][j] * DX[ix];
                    }
                    if (top && gate) {  // Dirichlet gate
                        vcoc = 0.; vcob = 0.;
                        for (int k = 0; k < 3; ++k) {
                            vcob = vcob - (cvy[i][k] - cxll[i][k] + cxrr[i][k]) * ep * acxrl[k][j] * DX[ix] / DY[jy];
                            vcoc = vcoc + (cvx[i][k] - cyll[i][k]) * ep * (acvx[k][j] + acyrr[k][j]) * DY[jy] / DX[ix] +
                                   (cvy[i][k] - cxll[i][k] + cxrr[i][k]) * ep * acvy[k][j] * DX[ix] / DY[jy] -
                                   cylr[i][k] * acyrl[k][j] * epr * DY[jy] / dxr;
                        }
                        vcob = vcob - c11 * cxrl[i][j] * DX[ix];
                        vcoc = vcoc + c11 * (cyrr[i][j] + cyll[i][j]) * DY[jy] + c11 * (cxrr[i][j] + cxll[i][j]) * DX[ix];
                    }
                    if (jy == NY - 1 && gate) {
                        vcott = 0.;
                        for (int k = 0; k < 3; ++k) vcott = vcott + cxlr[i][k] * ept * acvy[k][j] * DX[ix] / dyt;
                        vcott = vcott - c11 * cxlr[i][j] * DX[ix];
                    }
                    if (right) {  // Dirichlet right
                        vcoc = 0.; vcol = 0.;
                        for (int k = 0; k < 3; ++k) {
                            vcol = vcol - (cvx[i][k] - cyll[i][k] + cyrr[i][k]) * ep * acyrl[k][j] * DY[jy] / DX[ix];
                            if (!top)
                                vcoc = vcoc + (cvy[i][k] - cxll[i][k]) * ep * (acvy[k][j] + acxrr[k][j]) * DX[ix] / DY[jy] +
                                       (cvx[i][k] - cyll[i][k] + cyrr[i][k]) * ep * acvx[k][j] * DY[jy] / DX[ix] -
                                       cxlr[i][k] * acxrl[k][j] * ept * DX[ix] / dyt;
                            else
                                vcoc = vcoc + (cvy[i][k] - cxll[i][k]) * ep * (acvy[k][j] + acxrr[k][j]) * DX[ix] / DY[jy] +
                                       (cvx[i][k] - cyll[i][k] + cyrr[i][k]) * ep * acvx[k][j] * DY[jy] / DX[ix];
                        }
                        vcol = vcol - c11 * cyrl[i][j] * DY[jy];
                        if (!top)
                            vcoc = vcoc + c11 * (cyrr[i][j] + cyll[i][j]) * DY[jy] + c11 * (cxrr[i][j] + cxll[i][j]) * DX[ix];
                        else
                            vcoc = vcoc + c11 * (cyrr[i][j] + cyll[i][j]) * DY[jy] + c11 * cxll[i][j] * DX[ix];
                    }
                    if (ix == NX - 1) {
                        vcor = 0.;
                        for (int k = 0; k < 3; ++k) vcor = vcor + cylr[i][k] * acvx[k][j] * epr * DY[jy] / dxr;
                        vcor = vcor - c11 * cylr[i][j] * DY[jy];
                    }
                    if (jy == 1) {  // bottom
                        for (int k = 0; k < 3; ++k)
                            vcoc = vcoc - (cvy[i][k] - cxll[i][k]) * ep * (acvy[k][j] + acxrr[k][j]) * DX[ix] / DY[jy] +
                                   cvy[i][k] * ep * (acvy[k][j] + acxrr[k][j] - acxll[k][j]) * DX[ix] / DY[jy];
                        vcoc = vcoc - c11 * cxll[i][j] * DX[ix];
                    }
                    col[i][j] = vcol; cob[i][j] = vcob; coc[i][j] = vcoc; cott[i][j] = vcott; cor[i][j] = vcor;
                }
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) {
                    const int irow = (ii - 1) * 3 + j + 1;
                    int icol = (ii - 1) * 3 + k + 1;
                    ABP(irow - icol + m1, icol) = coc[j][k];
                    if (jy > 1) { icol = (ii - 2) * 3 + k + 1; ABP(irow - icol + m1, icol) = cob[j][k]; }
                    if (jy < NY) { icol = ii * 3 + k + 1; ABP(irow - icol + m1, icol) = cott[j][k]; }
                    if (ix < NX) { icol = (ii - 1 + NY) * 3 + k + 1; ABP(irow - icol + m1, icol) = cor[j][k]; }
                    if (ix > 1) { icol = (ii - 1 - NY) * 3 + k + 1; ABP(irow - icol + m1, icol) = col[j][k]; }
                }
        }
    int info = dgbtf2(ndim, ndim, nsub, nsuper, ps.ab.data(), ldab, ps.ipiv.data());
    if (info != 0) { err = "Poisson band matrix is singular"; return LP_ERR_INVALID; }
    return LP_OK;
}

}  // namespace

double weight_host(const Tables &t, int xi, int om) {
    const int n = t.n;
    int i = xi / (n * n), j = (xi / n) % n, k = xi % n;
    int l = om / (n * n), m = (om / n) % n, q = om % n;
    const double *s = &t.shat[6 * (size_t)om];
    double d0 = t.eta[i] - t.eta[l], d1 = t.eta[j] - t.eta[m], d2 = t.eta[k] - t.eta[q];
    double res = 0.;
    res += s[0] * d0 * d0; res += s[1] * d0 * d1; res += s[2] * d0 * d2;
    res += s[1] * d1 * d0; res += s[3] * d1 * d1; res += s[4] * d1 * d2;
    res += s[2] * d2 * d0; res += s[4] * d2 * d1; res += s[5] * d2 * d2;
    return t.rzero[om] ? -res : t.ahat[om] - res;
}

// The collision operator's tables: omega factors of the weight, conservation
// rows, node map, IntModes factors, DFT matrices, pair offsets, moment rows.
static lp_status build_collision_tables(const lp_params &p, Tables &t, std::string &err) {
    const int n = p.n, nv = p.nv;
    // Omega tables of gHat3 and the per-omega quadrature factor of ComputeQ
    // (C:745, C:804: prefactor*wtN[l]*wtN[m]*wtN[n] in that order).
    t.shat.resize(6 * (size_t)t.n3); t.ahat.resize(t.n3); t.rzero.resize(t.n3); t.cw.resize(t.n3);
    WeightFns W{t.PI, t.R_v};
    const double pre = t.h_eta * t.h_eta * t.h_eta;
    for (int o = 0; o < t.n3; ++o) {
        int l = o / (n * n), m = (o / n) % n, q = o % n;
        double k1 = t.eta[l], k2 = t.eta[m], k3 = t.eta[q];
        double r = std::sqrt(k1 * k1 + k2 * k2 + k3 * k3);
        double *s = &t.shat[6 * (size_t)o];
        s[0] = W.s1(k1, k2, k3) - W.s233(k2, k3, k1);
        s[3] = W.s1(k1, k2, k3) - W.s233(k1, k3, k2);
        s[5] = W.s1(k1, k2, k3) - W.s233(k1, k2, k3);
        s[1] = -W.s213(k1, k3, k2);
        s[2] = -W.s213(k1, k2, k3);
        s[4] = -W.s213(k2, k1, k3);
        t.rzero[o] = (r == 0.);
        t.ahat[o] = (r == 0.) ? 0. : (std::sqrt(8. / t.PI)) * (t.R_v * r - std::sin(t.R_v * r)) / (t.R_v * r);
        t.cw[o] = pre * t.wt[l] * t.wt[m] * t.wt[q];
    }

    // Conservation rows and inverse Gram matrix (K:133-209).
    t.c1.assign(5 * (size_t)t.n3, 0.); t.c2.assign(5 * (size_t)t.n3, 0.);
    const double L = t.L_v;
    const double *eta = t.eta.data();
    for (int ke = 0; ke < t.n3; ++ke) {
        int k = ke % n, j = ((ke - k) % (n * n)) / n, i = (ke - k - j * n) / (n * n);
        double a1, a2, a3;
        t.c1[0 * (size_t)t.n3 + ke] = sinc(L * eta[i]) * sinc(L * eta[j]) * sinc(L * eta[k]);
        if (eta[i] != 0) a1 = ((eta[i] * eta[i] * L * L - 2) * std::sin(eta[i] * L) + 2 * eta[i] * L * std::cos(eta[i] * L)) / (eta[i] * eta[i] * eta[i] * L);
        else a1 = L * L / 3.;
        if (eta[j] != 0) a2 = ((eta[j] * eta[j] * L * L - 2) * std::sin(eta[j] * L) + 2 * eta[j] * L * std::cos(eta[j] * L)) / (eta[j] * eta[j] * eta[j] * L);
        else a2 = L * L / 3.;
        if (eta[k] != 0) a3 = ((eta[k] * eta[k] * L * L - 2) * std::sin(eta[k] * L) + 2 * eta[k] * L * std::cos(eta[k] * L)) / (eta[k] * eta[k] * eta[k] * L);
        else a3 = L * L / 3.;
        t.c1[4 * (size_t)t.n3 + ke] = 0.5 * (a1 * sinc(L * eta[j]) * sinc(L * eta[k]) + a2 * sinc(L * eta[i]) * sinc(L * eta[k]) + a3 * sinc(L * eta[i]) * sinc(L * eta[j]));
        if (eta[i] != 0) t.c2[1 * (size_t)t.n3 + ke] = -sinc(L * eta[j]) * sinc(L * eta[k]) * (sinc(eta[i] * L) - std::cos(eta[i] * L)) / eta[i];
        if (eta[j] != 0) t.c2[2 * (size_t)t.n3 + ke] = -sinc(L * eta[i]) * sinc(L * eta[k]) * (sinc(eta[j] * L) - std::cos(eta[j] * L)) / eta[j];
        if (eta[k] != 0) t.c2[3 * (size_t)t.n3 + ke] = -sinc(L * eta[i]) * sinc(L * eta[j]) * (sinc(eta[k] * L) - std::cos(eta[k] * L)) / eta[k];
    }
    double cct[25];
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) {
            double s = 0.;
            for (int k = 0; k < t.n3; ++k)
                s += t.c1[(size_t)i * t.n3 + k] * t.c1[(size_t)j * t.n3 + k] + t.c2[(size_t)i * t.n3 + k] * t.c2[(size_t)j * t.n3 + k];
            cct[i * 5 + j] = s;
        }
    int piv[5];
    if (dgetf2(5, 5, cct, 5, piv) != 0 || dgetri(5, cct, 5, piv) != 0) {
        err = "conservation Gram matrix is singular";
        return LP_ERR_INVALID;
    }
    std::memcpy(t.cct_inv, cct, sizeof(cct));

    // Node -> DG cell map and node offsets v[l] - Gridv(j).
    t.nodecell.resize(n); t.nodeoff.resize(n);
    for (int l = 0; l < n; ++l) {
        int j = (int)((l * t.h_v) / t.dv);
        if (j == nv) j = nv - 1;
        t.nodecell[l] = j;
        t.nodeoff[l] = (t.v[l] - (-p.lv + ((double)j + 0.5) * t.dv)) / t.dv;
    }

    // Per-axis factors of IntModes (C:364-505).
    t.tfac.assign(2 * 3 * (size_t)n * nv, 0.);
    const double dv = t.dv;
    auto gridv = [&](double m) { return (-p.lv + (m + 0.5) * dv); };
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < nv; ++j) {
            double e = t.eta[k], gp = gridv(j + 0.5), gm = gridv(j - 0.5), gj = gridv((double)j);
            double t0r, t0i, t1r, t1i, t2r, t2i;
            if (e != 0.) {
                t0r = (std::sin(e * gp) - std::sin(e * gm)) / e;
                t0i = (std::cos(e * gm) - std::cos(e * gp)) / e;
                t1r = ((gp * std::sin(e * gp) - gm * std::sin(e * gm)) / e + (std::cos(e * gp) - std::cos(e * gm)) / e / e - gj * t0r) / dv;
                t1i = ((std::sin(e * gp) - std::sin(e * gm)) / e / e + (gm * std::cos(e * gm) - gp * std::cos(e * gp)) / e - gj * t0i) / dv;
                double ar = (gp * std::sin(e * gp) - gm * std::sin(e * gm)) / e + (std::cos(e * gp) - std::cos(e * gm)) / e / e;
                double aim = (std::sin(e * gp) - std::sin(e * gm)) / e / e + (gm * std::cos(e * gm) - gp * std::cos(e * gp)) / e;
                t2r = ((gp * gp * std::sin(e * gp) - gm * gm * std::sin(e * gm) - 2 * aim) / e - 2 * gj * ar + gj * gj * t0r) / dv / dv;
                t2i = ((gm * gm * std::cos(e * gm) - gp * gp * std::cos(e * gp) + 2 * ar) / e - 2 * gj * aim + gj * gj * t0i) / dv / dv;
            } else {
                t0r = dv; t0i = 0.; t1r = 0.; t1i = 0.; t2r = dv / 12.; t2i = 0.;
            }
            size_t b = (size_t)k * nv + j, st = (size_t)n * nv;
            t.tfac[2 * b] = t0r; t.tfac[2 * b + 1] = t0i;
            t.tfac[2 * (st + b)] = t1r; t.tfac[2 * (st + b) + 1] = t1i;
            t.tfac[2 * (2 * st + b)] = t2r; t.tfac[2 * (2 * st + b) + 1] = t2i;
        }

    // Moment functionals of the collided coefficients a = (U0, U3, U4, U5, U6)
    // of one record (MomentCalculations.cpp:3-47 divided by the cell volume
    // factors): mass a0 + a4/4; momentum_d G_d a0 + dv a_d/12 + G_d a4/4;
    // energy (|G|^2 + dv^2/4) a0 + dv/6 G.a + (19 dv^2/240 + |G|^2/4) a4.
    // Their exact increments are per-axis sums of the IntModes factors.
    {
        std::vector<double> S0(2 * n), S1(2 * n), S2(2 * n), SG0(2 * n), SG1(2 * n), SGG0(2 * n);
        for (int k = 0; k < n; ++k)
            for (int j = 0; j < nv; ++j) {
                const double g = gridv((double)j);
                const size_t b = (size_t)k * nv + j, st = (size_t)n * nv;
                for (int ri = 0; ri < 2; ++ri) {
                    const double t0 = t.tfac[2 * b + ri], t1 = t.tfac[2 * (st + b) + ri], t2 = t.tfac[2 * (2 * st + b) + ri];
                    S0[2 * k + ri] += t0; S1[2 * k + ri] += t1; S2[2 * k + ri] += t2;
                    SG0[2 * k + ri] += g * t0; SG1[2 * k + ri] += g * t1; SGG0[2 * k + ri] += g * g * t0;
                }
            }
        auto cm = [](const double *a, const double *b, double *o) {
            o[0] = a[0] * b[0] - a[1] * b[1];
            o[1] = a[0] * b[1] + a[1] * b[0];
        };
        auto triple = [&](const double *a, const double *b, const double *c3, double *o) {
            double ab[2];
            cm(a, b, ab);
            cm(ab, c3, o);
        };
        t.gmom.assign(2 * 5 * (size_t)t.n3, 0.);
        for (int ke = 0; ke < t.n3; ++ke) {
            const int k1 = ke / (n * n), k2 = (ke / n) % n, k3 = ke % n;
            const double *s0[3] = {&S0[2 * k1], &S0[2 * k2], &S0[2 * k3]};
            double g[5][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}}, tmp[2];
            triple(s0[0], s0[1], s0[2], g[0]);
            const int kk[3] = {k1, k2, k3};
            for (int d = 0; d < 3; ++d) {
                double fac[2] = {SG0[2 * kk[d]] + t.dv * S1[2 * kk[d]], SG0[2 * kk[d] + 1] + t.dv * S1[2 * kk[d] + 1]};
                double efac[2] = {SGG0[2 * kk[d]] + t.dv * t.dv * S2[2 * kk[d]] + 2 * t.dv * SG1[2 * kk[d]],
                                  SGG0[2 * kk[d] + 1] + t.dv * t.dv * S2[2 * kk[d] + 1] + 2 * t.dv * SG1[2 * kk[d] + 1]};
                const double *o1 = s0[(d + 1) % 3], *o2 = s0[(d + 2) % 3];
                triple(fac, o1, o2, tmp);
                g[1 + d][0] = tmp[0]; g[1 + d][1] = tmp[1];
                triple(efac, o1, o2, tmp);
                g[4][0] += tmp[0]; g[4][1] += tmp[1];
            }
            for (int m = 0; m < 5; ++m) {
                t.gmom[2 * ((size_t)m * t.n3 + ke)] = g[m][0];
                t.gmom[2 * ((size_t)m * t.n3 + ke) + 1] = g[m][1];
            }
        }
        double gm[25] = {0};
        for (int j1 = 0; j1 < nv; ++j1)
            for (int j2 = 0; j2 < nv; ++j2)
                for (int j3 = 0; j3 < nv; ++j3) {
                    const double G[3] = {gridv((double)j1), gridv((double)j2), gridv((double)j3)};
                    const double g2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
                    double Phi[5][5] = {{1, 0, 0, 0, 0.25},
                                        {G[0], dv / 12., 0, 0, G[0] / 4.},
                                        {G[1], 0, dv / 12., 0, G[1] / 4.},
                                        {G[2], 0, 0, dv / 12., G[2] / 4.},
                                        {g2 + dv * dv / 4., dv * G[0] / 6., dv * G[1] / 6., dv * G[2] / 6.,
                                         19. * dv * dv / 240. + g2 / 4.}};
                    for (int a = 0; a < 5; ++a)
                        for (int b = 0; b < 5; ++b)
                            for (int q = 0; q < 5; ++q) gm[a * 5 + b] += Phi[a][q] * Phi[b][q];
                }
        int gp[5];
        if (dgetf2(5, 5, gm, 5, gp) != 0 || dgetri(5, gm, 5, gp) != 0) {
            err = "moment Gram matrix is singular";
            return LP_ERR_INVALID;
        }
        std::memcpy(t.gm_inv, gm, sizeof(gm));
    }

    // Per-axis DFT matrices with the phases and scalings of fft3D (C:163-197)
    // and FS (C:241-276) folded in.  Forward: out[a] = sum_i M[a][i] in[i].
    t.mfwd.assign(2 * (size_t)n * n, 0.); t.minv.assign(2 * (size_t)n * n, 0.);
    const double inv_s = 1.0 / (2.0 * t.L_v * t.scale);
    for (int a = 0; a < n; ++a)
        for (int i = 0; i < n; ++i) {
            double ang = (double)i * t.L_eta * t.h_v + t.L_v * t.eta[a] -
                         2.0 * t.PI * (double)(((long)a * i) % n) / (double)n;
            double mag = t.scale * t.h_v * t.wt[i];
            t.mfwd[2 * ((size_t)a * n + i)] = mag * std::cos(ang);
            t.mfwd[2 * ((size_t)a * n + i) + 1] = mag * std::sin(ang);
            // inverse: output node a (velocity), input mode i
            double angi = -(double)i * t.L_v * t.h_eta + 2.0 * t.PI * (double)(((long)a * i) % n) / (double)n -
                          t.L_eta * t.v[a];
            t.minv[2 * ((size_t)a * n + i)] = inv_s * std::cos(angi);
            t.minv[2 * ((size_t)a * n + i) + 1] = inv_s * std::sin(angi);
        }

    // The matrices' factors: the DFT core w^(a i) between a phase (and
    // trapezoid weight) on the input index and a phase on the output index.
    for (int d = 0; d < 2; ++d) {
        t.dpre[d].assign(2 * (size_t)n, 0.); t.dpost[d].assign(2 * (size_t)n, 0.); t.dw[d].assign(2 * (size_t)n, 0.);
    }
    for (int i = 0; i < n; ++i) {
        const double pf = (double)i * t.L_eta * t.h_v, mf = t.scale * t.h_v * t.wt[i];
        t.dpre[0][2 * i] = mf * std::cos(pf); t.dpre[0][2 * i + 1] = mf * std::sin(pf);
        const double pi_ = -(double)i * t.L_v * t.h_eta;
        t.dpre[1][2 * i] = inv_s * std::cos(pi_); t.dpre[1][2 * i + 1] = inv_s * std::sin(pi_);
        const double of = t.L_v * t.eta[i], oi = -t.L_eta * t.v[i];
        t.dpost[0][2 * i] = std::cos(of); t.dpost[0][2 * i + 1] = std::sin(of);
        t.dpost[1][2 * i] = std::cos(oi); t.dpost[1][2 * i + 1] = std::sin(oi);
        const double wk = 2.0 * t.PI * (double)i / (double)n;
        t.dw[0][2 * i] = std::cos(wk); t.dw[0][2 * i + 1] = -std::sin(wk);
        t.dw[1][2 * i] = std::cos(wk); t.dw[1][2 * i + 1] = std::sin(wk);
    }
    {
        double dev = 0., big = 0.;
        for (int d = 0; d < 2; ++d) {
            const std::vector<double> &M = d == 0 ? t.mfwd : t.minv;
            for (int a = 0; a < n; ++a)
                for (int i = 0; i < n; ++i) {
                    const int k = (int)(((long)a * i) % n);
                    const double *po = &t.dpost[d][2 * a], *w = &t.dw[d][2 * k], *pr = &t.dpre[d][2 * i];
                    const double xr = po[0] * w[0] - po[1] * w[1], xi = po[0] * w[1] + po[1] * w[0];
                    const double yr = xr * pr[0] - xi * pr[1], yi = xr * pr[1] + xi * pr[0];
                    const size_t o = 2 * ((size_t)a * n + i);
                    dev = std::max(dev, std::max(std::fabs(yr - M[o]), std::fabs(yi - M[o + 1])));
                    big = std::max(big, std::max(std::fabs(M[o]), std::fabs(M[o + 1])));
                }
        }
        t.dft_fac_ok = dev <= 1e-12 * big;
    }

    // Pair table offsets: for xi, the window of omega is a box symmetric under
    // omega -> xi + n/2 - omega; it has ceil(cnt/2) pairs.
    t.pair_off.assign(t.n3 + 1, 0);
    const int h = n / 2;
    for (int xi = 0; xi < t.n3; ++xi) {
        int i = xi / (n * n), j = (xi / n) % n, k = xi % n;
        int ni = i < h ? i + h + 1 : 3 * h - 1 - i;
        int nj = j < h ? j + h + 1 : 3 * h - 1 - j;
        int nk = k < h ? k + h + 1 : 3 * h - 1 - k;
        int cnt = ni * nj * nk;
        t.pair_off[xi + 1] = t.pair_off[xi] + (cnt + 1) / 2;
    }
    if (p.linear_ei) {
        t.win_off.assign(t.n3 + 1, 0);
        for (int xi = 0; xi < t.n3; ++xi) {
            int i = xi / (n * n), j = (xi / n) % n, k = xi % n;
            long long cnt = (long long)(i < h ? i + h + 1 : 3 * h - 1 - i) * (j < h ? j + h + 1 : 3 * h - 1 - j) *
                            (k < h ? k + h + 1 : 3 * h - 1 - k);
            t.win_off[xi + 1] = t.win_off[xi] + cnt;
        }
        // CCt_linear (K:190-199): Gram matrix of rows C1[0], C1[4], inverted
        double g[4] = {0, 0, 0, 0};
        for (int k = 0; k < t.n3; ++k) {
            g[0] += t.c1[0 * (size_t)t.n3 + k] * t.c1[0 * (size_t)t.n3 + k] + t.c2[0 * (size_t)t.n3 + k] * t.c2[0 * (size_t)t.n3 + k];
            g[1] += t.c1[0 * (size_t)t.n3 + k] * t.c1[4 * (size_t)t.n3 + k] + t.c2[0 * (size_t)t.n3 + k] * t.c2[4 * (size_t)t.n3 + k];
            g[3] += t.c1[4 * (size_t)t.n3 + k] * t.c1[4 * (size_t)t.n3 + k] + t.c2[4 * (size_t)t.n3 + k] * t.c2[4 * (size_t)t.n3 + k];
        }
        g[2] = g[1];
        int piv2[2];
        if (dgetf2(2, 2, g, 2, piv2) != 0 || dgetri(2, g, 2, piv2) != 0) {
            err = "two-species Gram matrix is singular";
            return LP_ERR_INVALID;
        }
        std::fill(t.cct_lin5, t.cct_lin5 + 25, 0.);
        t.cct_lin5[0 * 5 + 0] = g[0]; t.cct_lin5[0 * 5 + 4] = g[1];
        t.cct_lin5[4 * 5 + 0] = g[2]; t.cct_lin5[4 * 5 + 4] = g[3];
    }

    return LP_OK;
}

lp_status build_tables(const lp_params &p, Tables &t, std::string &err, unsigned parts) {
    if (p.nx1 < 2 || p.nx2 < 1 || p.nv < 2 || p.n < 4 || (p.n % 2) != 0 || p.n > 32) {
        err = "need nx1 >= 2, nx2 >= 1, nv >= 2 and an even n in [4, 32]";
        return LP_ERR_INVALID;
    }
    if (!(p.lv > 0) || !(p.lx > 0) || !(p.dt > 0) || p.nu < 0 || !(p.k_wave > 0)) {
        err = "need lv, lx, dt, k_wave > 0 and nu >= 0";
        return LP_ERR_INVALID;
    }
    if ((long long)p.nx1 * p.nx2 * p.nv * p.nv * p.nv * 7 > (1LL << 40)) {
        err = "state too large";
        return LP_ERR_INVALID;
    }
    if (p.precision != LP_PREC_FP64 && p.precision != LP_PREC_MIXED) {
        err = "unknown precision";
        return LP_ERR_INVALID;
    }
    t.prm = p;
    t.n = p.n; t.nv = p.nv;
    t.n3 = p.n * p.n * p.n;
    t.nv3 = p.nv * p.nv * p.nv;
    t.ncell = p.nx1 * p.nx2;
    t.size = (long long)t.ncell * t.nv3;
    t.ncollide = (p.fixes & LP_FIX_F3) ? t.ncell : std::min(p.nx1, t.ncell);
    // Grids and constants (M:38-40, M:66, M:270-284).
    t.PI = M_PI;
    t.dv = 2. * p.lv / p.nv;
    t.dx = p.lx / p.nx1;
    t.dy = p.lx / p.nx2;
    t.scaleL = 8 * p.lv * p.lv * p.lv;
    t.scalev = t.dv * t.dv * t.dv;
    t.scale = 1.0 / std::sqrt(2.0 * M_PI);
    t.scale3 = std::pow(t.scale, 3.0);
    t.L_v = p.lv; t.R_v = p.lv;
    t.L_eta = 0.5 * (double)(p.n - 1) * t.PI / t.L_v;
    t.h_v = 2.0 * t.L_v / (double)(p.n - 1);
    t.h_eta = 2.0 * t.L_eta / (double)(p.n);
    const int n = p.n, nv = p.nv;
    t.v.resize(n); t.eta.resize(n); t.wt.assign(n, 1.0);
    for (int i = 0; i < n; ++i) {
        t.eta[i] = -t.L_eta + (double)i * t.h_eta;
        t.v[i] = -t.L_v + (double)i * t.h_v;
    }
    if ((p.fixes & LP_FIX_F11) && std::fabs(t.eta[n / 2]) < 1e-12 * t.L_eta) t.eta[n / 2] = 0.;
    t.wt[0] = 0.5; t.wt[n - 1] = 0.5;  // trapezoidalRule

    if (parts & kTablesCollision) {
        const lp_status s = build_collision_tables(p, t, err);
        if (s != LP_OK) return s;
    }
    if (!(parts & kTablesPoisson)) return LP_OK;
    return build_poisson(t, err);
}


// Columns of A^-1 by the band solve of DGBTRS ('N') with the factors of
// build_poisson: forward elimination with the row interchanges, then the
// banded upper-triangular back substitution.
void poisson_inverse(const PoissonTables &ps, std::vector<double> &inv) {
    const int n = ps.ndim, kl = ps.kl, ku = ps.ku, ldab = ps.ldab, kd = ku + kl + 1, k = kl + ku;
    auto AB = [&](int i, int j) { return ps.ab[(size_t)(i - 1) + (size_t)(j - 1) * ldab]; };
    inv.assign((size_t)n * n, 0.);
    std::vector<double> b(n);
    for (int col = 0; col < n; ++col) {
        std::fill(b.begin(), b.end(), 0.);
        b[col] = 1.;
        for (int j = 1; j <= n - 1; ++j) {
            const int lm = std::min(kl, n - j), l = ps.ipiv[j - 1];
            if (l != j) std::swap(b[l - 1], b[j - 1]);
            const double bj = b[j - 1];
            if (bj != 0.)
                for (int i = 1; i <= lm; ++i) b[j + i - 1] -= AB(kd + i, j) * bj;
        }
        for (int j = n; j >= 1; --j) {
            if (b[j - 1] == 0.) continue;
            const double xj = b[j - 1] / AB(k + 1, j);
            b[j - 1] = xj;
            for (int i = std::max(1, j - k); i <= j - 1; ++i) b[i - 1] -= xj * AB(k + 1 - j + i, j);
        }
        for (int r = 0; r < n; ++r) inv[(size_t)r * n + col] = b[r];
    }
}

}  // namespace lp
