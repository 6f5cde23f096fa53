// exfem_oracle.cpp — CPU oracle for the explicit time loop of damian.par.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, in plain FP64 C++, what the
// reference's Fortran does on one MPI rank, so that the CUDA library can be
// checked against it.  It is linked only by tests/, __graft_entry__.smoke()
// and the cpu_baseline / --impl reference legs of bench.py; the product never
// calls it.
//
// Parity status: the reference cannot be built in this environment (no
// gfortran/MPI/ParMETIS/ACML, and model.f90:643 assigns the undeclared `red`),
// and its tests hold no golden vectors for this path, so this restatement is
// pinned by mathematical known-answer tests and by the reference's own io.cpp
// (file formats) only: parity unpinned against a reference run.
//
// What it follows, line by line (damian.par file:line):
//   setupconstants        explicit.f90:72-77
//   init_explicit         explicit.f90:79-109
//   run_explicit          explicit.f90:111-159 (element loop 129-142; the
//                         dgemv('N',8,8,-1,K,8,u,1,1,r,1) of 139-140 in the
//                         column order of the reference BLAS)
//   elemallnhnodes/dofs   model.f90:126-133, 163-174
//   elength/getmassof     model.f90:112-118, 564-577; calcm formulation.f90:250-254
//   getdampingof/lysmer   model.f90:585-604; formulation.f90:219-229
//   sum_reactanchors      model.f90:632-647 (literal text, `red` as real*8(2)),
//                         or the halving twin of communicator.f90:1232
//   set_dispshanging      model.f90:612-624
//   wave_reactions        model.f90:745-800; multdrm formulation.f90:378-393
//   calck / calcsqm       formulation.f90:276-313, 256-268
//   initplanewaves/wavep/wavesv  pwaves.f90:16-98, 148-217
//   visu_field/shapes     visualization.f90:156-181; formulation.f90:315-363
//   inside_soil           model.f90:217-235; tolerances utilities.f90:159-175
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "exfem_gpu.h"

namespace {

constexpr double U_PI = 3.14159265358979323846;
constexpr double U_TOL = 1.0e-9;
// f_wangzero = 0.0001 is a default-kind (single) literal stored in a real*8
// parameter (pwaves.f90:8).
const double F_WANGZERO = (double)0.0001f;

inline bool realunder(double a, double b) { return (a - b) < -U_TOL; }
inline bool realover(double a, double b) { return (a - b) > U_TOL; }

std::string g_err;

// ---------------------------------------------------------------- pwaves --
struct PWave {
    int kind = 0;
    double walpha = 0, wbeta = 0, wfreq = 0;
    double wsine = 0, wcose = 0, wsinf = 0, wcosf = 0;
    double wa = 0, wa1 = 0, wb = 0, wb1 = 0;
    double wui[2][3] = {{0, 0, 0}, {0, 0, 0}};   // f_wui(2,3) as wui[row-1][col-1]
};

// initplanewaves (pwaves.f90:16-98); returns EXFEM_E_UNSUPPORTED where the
// reference calls exit(1).
int initplanewaves(PWave &w, int kind, double mag, double alpha, double beta, double angle, double freq) {
    w = PWave();
    w.kind = kind;
    w.walpha = alpha;
    w.wbeta = beta;
    w.wfreq = freq;
    if (kind == EXFEM_WAVE_P) {
        double e = angle, a = mag;
        w.wsine = std::sin(e);
        w.wsinf = w.wsine * (beta / alpha);
        double f = std::asin(w.wsinf);
        w.wcose = std::cos(e);
        w.wcosf = std::cos(f);
        if (w.wcose < F_WANGZERO) {
            g_err = "Grazing incidence. Not implemented.";
            return EXFEM_E_UNSUPPORTED;
        } else if (std::fabs(w.wsine) < F_WANGZERO) {
            w.wa = a;
            w.wa1 = -w.wa;
            w.wb1 = 0.0;
            w.wcose = 1;
            w.wsine = 0;
        } else {
            double sin2e = std::sin(2 * e), sin2f = std::sin(2 * f), cos2f = std::cos(2 * f);
            double r = alpha / beta;
            w.wa = a;
            w.wa1 = (sin2e * sin2f - (r * r) * (cos2f * cos2f));
            w.wa1 = w.wa1 / (sin2e * sin2f + (r * r) * (cos2f * cos2f));
            w.wa1 = w.wa1 * a;
            w.wb1 = -(2 * r * sin2e * cos2f);
            w.wb1 = w.wb1 / (sin2e * sin2f + (r * r) * (cos2f * cos2f));
            w.wb1 = w.wb1 * a;
        }
        w.wui[0][0] = w.wsine;  w.wui[1][0] = -w.wcose;
        w.wui[0][1] = w.wsine;  w.wui[1][1] = w.wcose;
        w.wui[0][2] = -w.wcosf; w.wui[1][2] = w.wsinf;
    } else if (kind == EXFEM_WAVE_SV) {
        double f = angle, b = mag;
        w.wsinf = std::sin(f);
        double fcr = std::asin(beta / alpha);
        w.wsine = w.wsinf * (alpha / beta);
        double e = std::asin(w.wsine);
        w.wcose = std::cos(e);
        w.wcosf = std::cos(f);
        if (std::fabs(w.wsinf) < F_WANGZERO) {
            w.wb = b;
            w.wb1 = -w.wb;
            w.wa1 = 0.0;
            w.wcosf = 1;
            w.wsinf = 0;
        } else if ((fcr - f) > F_WANGZERO) {
            double sin2e = std::sin(2 * e), sin2f = std::sin(2 * f), cos2f = std::cos(2 * f);
            double r = alpha / beta;
            w.wb = b;
            w.wb1 = (sin2e * sin2f - (r * r) * (cos2f * cos2f));
            w.wb1 = w.wb1 / (sin2e * sin2f + (r * r) * (cos2f * cos2f));
            w.wb1 = w.wb1 * b;
            w.wa1 = r * std::sin(4.0 * f);
            w.wa1 = w.wa1 / (sin2e * sin2f + (r * r) * (cos2f * cos2f));
            w.wa1 = w.wa1 * b;
        } else {
            g_err = "Inhomogeneous waves. Not implemented";
            return EXFEM_E_UNSUPPORTED;
        }
        w.wui[0][0] = w.wcosf;  w.wui[1][0] = w.wsinf;
        w.wui[0][1] = w.wsine;  w.wui[1][1] = w.wcose;
        w.wui[0][2] = -w.wcosf; w.wui[1][2] = w.wsinf;
    } else {
        g_err = "unknown wave kind";
        return EXFEM_E_ARG;
    }
    return 0;
}

// One Ricker term and its two time derivatives (the three columns of
// ip/rp/rs in wavep/wavesv, pwaves.f90:157-169, 193-205).
inline void ricker3(double freq, double t, double v, double out[3]) {
    double fp = freq * U_PI;
    double d = t - v;
    double q = fp * d;
    double v2 = q * q;
    double e = std::exp(v2);
    out[0] = (1.0 - 2.0 * v2) / e;
    out[1] = (2.0 * v2 - 3.0) * (fp * fp) * d / e;
    out[2] = -2.0 * (4.0 * (v2 * v2) - 12.0 * v2 + 3.0) * (fp * fp) / e;
}

// planewave (pwaves.f90:100-111): u[comp][col], comp = x/z, col = u/du/ddu.
void planewave(const PWave &w, double t, double x1, double x3, double u[2][3]) {
    double v[3];
    double amp0;
    if (w.kind == EXFEM_WAVE_P) {
        v[0] = (x1 * w.wsine - x3 * w.wcose) / w.walpha;
        amp0 = w.wa;
    } else {
        v[0] = (x1 * w.wsinf - x3 * w.wcosf) / w.wbeta;
        amp0 = w.wb;
    }
    v[1] = (x1 * w.wsine + x3 * w.wcose) / w.walpha;
    v[2] = (x1 * w.wsinf + x3 * w.wcosf) / w.wbeta;
    double r0[3], r1[3], r2[3];
    ricker3(w.wfreq, t, v[0], r0);
    ricker3(w.wfreq, t, v[1], r1);
    ricker3(w.wfreq, t, v[2], r2);
    for (int c = 0; c < 3; ++c) {
        double ipx = r0[c] * w.wui[0][0] * amp0, ipz = r0[c] * w.wui[1][0] * amp0;
        double rpx = r1[c] * w.wui[0][1] * w.wa1, rpz = r1[c] * w.wui[1][1] * w.wa1;
        double rsx = r2[c] * w.wui[0][2] * w.wb1, rsz = r2[c] * w.wui[1][2] * w.wb1;
        u[0][c] = ipx + rpx + rsx;
        u[1][c] = ipz + rpz + rsz;
    }
}

// calck (formulation.f90:276-313), column-major k[col*8+row].
void calck(double m, double l, double *k) {
    const double v[64] = {
        (3.0 * m + l) / 3.0, (m + l) / 4.0, -(3.0 * m + 2.0 * l) / 6.0, -(m - l) / 4.0,
        -(3.0 * m + l) / 6.0, -(m + l) / 4.0, l / 6.0, (m - l) / 4.0,
        (m + l) / 4.0, (3.0 * m + l) / 3.0, (m - l) / 4.0, l / 6.0,
        -(m + l) / 4.0, -(3.0 * m + l) / 6.0, -(m - l) / 4.0, -(3.0 * m + 2.0 * l) / 6.0,
        -(3.0 * m + 2.0 * l) / 6.0, (m - l) / 4.0, (3.0 * m + l) / 3.0, -(m + l) / 4.0,
        l / 6.0, -(m - l) / 4.0, -(3.0 * m + l) / 6.0, (m + l) / 4.0,
        -(m - l) / 4.0, l / 6.0, -(m + l) / 4.0, (3.0 * m + l) / 3.0,
        (m - l) / 4.0, -(3.0 * m + 2.0 * l) / 6.0, (m + l) / 4.0, -(3.0 * m + l) / 6.0,
        -(3.0 * m + l) / 6.0, -(m + l) / 4.0, l / 6.0, (m - l) / 4.0,
        (3.0 * m + l) / 3.0, (m + l) / 4.0, -(3.0 * m + 2.0 * l) / 6.0, -(m - l) / 4.0,
        -(m + l) / 4.0, -(3.0 * m + l) / 6.0, -(m - l) / 4.0, -(3.0 * m + 2.0 * l) / 6.0,
        (m + l) / 4.0, (3.0 * m + l) / 3.0, (m - l) / 4.0, l / 6.0,
        l / 6.0, -(m - l) / 4.0, -(3.0 * m + l) / 6.0, (m + l) / 4.0,
        -(3.0 * m + 2.0 * l) / 6.0, (m - l) / 4.0, (3.0 * m + l) / 3.0, -(m + l) / 4.0,
        (m - l) / 4.0, -(3.0 * m + 2.0 * l) / 6.0, (m + l) / 4.0, -(3.0 * m + l) / 6.0,
        -(m - l) / 4.0, l / 6.0, -(m + l) / 4.0, (3.0 * m + l) / 3.0};
    std::memcpy(k, v, sizeof(v));
}

// calcsqm (formulation.f90:256-268)
void calcsqm(double *m) {
    const double v[64] = {4, 0, 2, 0, 1, 0, 2, 0, 0, 4, 0, 2, 0, 1, 0, 2, 2, 0, 4, 0, 2, 0, 1, 0,
                          0, 2, 0, 4, 0, 2, 0, 1, 1, 0, 2, 0, 4, 0, 2, 0, 0, 1, 0, 2, 0, 4, 0, 2,
                          2, 0, 1, 0, 2, 0, 4, 0, 0, 2, 0, 1, 0, 2, 0, 4};
    for (int i = 0; i < 64; ++i) m[i] = v[i] / 9.0;
}

// multdrm (formulation.f90:378-393)
void multdrm(const double *k, const double *u, const bool *e, double *p) {
    for (int i = 0; i < 8; ++i) p[i] = 0.0;
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j)
            if (e[j] && !e[i]) {
                p[i] = p[i] - k[j * 8 + i] * u[j];
                p[j] = p[j] + k[i * 8 + j] * u[i];
            }
}

void drm_mask(int bck, bool e[8]) {  // model.f90:778-793
    static const bool SVERL[8] = {1, 1, 0, 0, 0, 0, 1, 1};
    static const bool SVERR[8] = {0, 0, 1, 1, 1, 1, 0, 0};
    static const bool SHORI[8] = {0, 0, 0, 0, 1, 1, 1, 1};
    static const bool CORNL[8] = {1, 1, 0, 0, 1, 1, 1, 1};
    static const bool CORNR[8] = {0, 0, 1, 1, 1, 1, 1, 1};
    const bool *src = nullptr;
    switch (bck) {
        case 2: src = SVERL; break;
        case 4: src = SVERR; break;
        case 1: src = SHORI; break;
        case 6: src = CORNL; break;
        case 5: src = CORNR; break;
        default: break;
    }
    for (int i = 0; i < 8; ++i) e[i] = src ? src[i] : false;
}

// ricker (formulation.f90:53-59): the point-source pulse.
double ricker_point(double amp, double sigma, double t) {
    double r = std::exp(-(t * t) / (4 * sigma)) * (t * t - 2 * sigma) / (8 * std::sqrt(U_PI) * std::pow(sigma, 2.5));
    return r * amp;
}

struct Solver {
    const exfem_mesh *mesh;
    const exfem_problem *prob;
    int nn, ne;
    double dt;
    double ea[4];
    std::vector<double> kmat;   // 64 * nmat
    double mmat[64];
    std::vector<double> mfull, u, up, ro;
    PWave wave;
    bool have_wave = true;   // false: no plane wave (point-source problems), no free field
    double t0 = 0;
    int hang_mode = EXFEM_HANG_HALF;
    std::vector<int> pdofs;  // y dof (0-based) of each point-source node, unique

    // elemallnhnodes (1-based node ids)
    inline void elemallnhnodes(int ele, int nodes[4]) const {
        int k = 0;
        for (int j = mesh->eptr[ele] - 1; j < mesh->eptr[ele + 1] - 1; ++j)
            if (!mesh->ediv[j]) { if (k < 4) nodes[k] = mesh->eind[j]; ++k; }
    }
    inline void elemallnhdofs(int ele, int dofs[8]) const {   // 1-based dofs
        int nodes[4];
        elemallnhnodes(ele, nodes);
        for (int k = 0; k < 4; ++k) { dofs[2 * k] = nodes[k] * 2 - 1; dofs[2 * k + 1] = dofs[2 * k] + 1; }
    }
    inline double elength(int ele) const {
        int nodes[4];
        elemallnhnodes(ele, nodes);
        return mesh->nodes[2 * (nodes[2] - 1) + 1] - mesh->nodes[2 * (nodes[0] - 1) + 1];
    }
    inline double getmassof(int ele) const {
        double scl = elength(ele) / 2.0;
        return (scl * scl) * prob->matconst[5 * (mesh->ematprop[ele] - 1) + 2];
    }
    inline void getdampingof(int ele, double damping[8]) const {
        int epr = mesh->ematprop[ele] - 1;
        const double *mc = &prob->matconst[5 * epr];
        for (int i = 0; i < 8; ++i) damping[i] = 0.0;
        int nodes[4];
        elemallnhnodes(ele, nodes);
        for (int i = 0; i < 4; ++i) {
            int ab = prob->absorbing[nodes[i] - 1];
            if (ab == 1 || ab == 2) {
                double scl = elength(ele), rho = mc[2];
                double r0 = mc[3] * rho * scl, r1 = mc[4] * rho * scl;
                if (ab == 1) { damping[2 * i] = r1; damping[2 * i + 1] = r0; }   // AB_ZDIR swaps
                else { damping[2 * i] = r0; damping[2 * i + 1] = r1; }
            }
        }
    }
    void sum_reactanchors(std::vector<double> &v) const {
        for (int i = 0; i < prob->nhanging; ++i) {
            const int *hg = &prob->hanging[3 * i];
            int dh = 2 * hg[0] - 2, da = 2 * hg[1] - 2, db = 2 * hg[2] - 2;
            double red[2];
            for (int c = 0; c < 2; ++c) {
                if (hang_mode == EXFEM_HANG_LITERAL) red[c] = v[dh + c] - (v[da + c] + v[db + c]) / 2.0;
                else red[c] = v[dh + c] / 2.0;
            }
            for (int c = 0; c < 2; ++c) v[da + c] = v[da + c] + red[c];
            for (int c = 0; c < 2; ++c) v[db + c] = v[db + c] + red[c];
        }
    }
    void set_dispshanging(std::vector<double> &v) const {
        for (int i = 0; i < prob->nhanging; ++i) {
            const int *hg = &prob->hanging[3 * i];
            int dh = 2 * hg[0] - 2, da = 2 * hg[1] - 2, db = 2 * hg[2] - 2;
            for (int c = 0; c < 2; ++c) v[dh + c] = (v[da + c] + v[db + c]) / 2.0;
        }
    }
    bool inside_soil(double x, double y) const {
        return realunder(x, prob->wbox[0]) || realover(x, prob->wbox[1]) || realover(y, prob->wbox[2]);
    }
    void wave_reactions(double time, std::vector<double> &r) const {
        double outt = time - t0;   // timetransform
        for (int s = 0; s < prob->nseismic; ++s) {
            int ele = prob->seismic[2 * s] - 1, bck = prob->seismic[2 * s + 1];
            int nodes[4], edofs[8];
            elemallnhnodes(ele, nodes);
            elemallnhdofs(ele, edofs);
            double mass = getmassof(ele);
            double uu[8], aa[8], p[8];
            for (int j = 0; j < 4; ++j) {
                double ox = mesh->nodes[2 * (nodes[j] - 1)] - prob->worigin[0];
                double oz = mesh->nodes[2 * (nodes[j] - 1) + 1] - prob->worigin[1];
                double up6[2][3];
                planewave(wave, outt, ox, oz, up6);
                uu[2 * j] = up6[0][0]; uu[2 * j + 1] = up6[1][0];
                aa[2 * j] = up6[0][2]; aa[2 * j + 1] = up6[1][2];
            }
            bool e[8];
            drm_mask(bck, e);
            multdrm(&kmat[64 * (mesh->ematprop[ele] - 1)], uu, e, p);
            for (int k = 0; k < 8; ++k) r[edofs[k] - 1] = r[edofs[k] - 1] + p[k];
            multdrm(mmat, aa, e, p);
            for (int k = 0; k < 8; ++k) p[k] = p[k] * mass;
            for (int k = 0; k < 8; ++k) r[edofs[k] - 1] = r[edofs[k] - 1] + p[k];
        }
    }
    // element term of explicit.f90:130-140 into localr
    inline void element_term(int j, double localr[8], int dofs[8]) const {
        elemallnhdofs(j, dofs);
        double mass = getmassof(j);
        double damping[8];
        getdampingof(j, damping);
        double localu[8], localup[8];
        for (int k = 0; k < 8; ++k) { localu[k] = u[dofs[k] - 1]; localup[k] = up[dofs[k] - 1]; }
        for (int k = 0; k < 8; ++k) localr[k] = (ea[2] * localu[k] - ea[0] * localup[k]) * mass;
        for (int k = 0; k < 8; ++k) localr[k] = localr[k] + ea[1] * damping[k] * localup[k];
        // dgemv('N', 8, 8, -1.0, K, 8, localu, 1, 1.0, localr, 1), reference BLAS order
        const double *K = &kmat[64 * (mesh->ematprop[j] - 1)];
        for (int c = 0; c < 8; ++c) {
            double temp = -1.0 * localu[c];
            for (int r = 0; r < 8; ++r) localr[r] = localr[r] + temp * K[c * 8 + r];
        }
    }
    void sample(int save, std::vector<double> &out, int nrecv) const {
        double time = dt * (double)save * (double)prob->io_interval;
        for (int i = 0; i < nrecv; ++i) {
            int ele = prob->recv_elem[i] - 1;
            double px = prob->recv_xy[2 * i], py = prob->recv_xy[2 * i + 1];
            int nodes[4], dofs[8];
            elemallnhnodes(ele, nodes);
            elemallnhdofs(ele, dofs);
            double x1 = mesh->nodes[2 * (nodes[0] - 1)], y1 = mesh->nodes[2 * (nodes[0] - 1) + 1];
            double x3 = mesh->nodes[2 * (nodes[2] - 1)], y3 = mesh->nodes[2 * (nodes[2] - 1) + 1];
            double r = (px - x1) / (x3 - x1), s = (py - y1) / (y3 - y1);
            r = 2.0 * r - 1.0; s = 2.0 * s - 1.0;
            r = std::max(-1.0, r); s = std::max(-1.0, s);
            r = std::min(1.0, r); s = std::min(1.0, s);
            double inter[4] = {(1 - r) * (1 - s) / 4, (1 + r) * (1 - s) / 4, (1 + r) * (1 + s) / 4, (1 - r) * (1 + s) / 4};
            double fx = 0.0, fy = 0.0;
            for (int k = 0; k < 4; ++k) {
                fx = fx + inter[k] * u[dofs[2 * k] - 1];
                fy = fy + inter[k] * u[dofs[2 * k + 1] - 1];
            }
            if (have_wave && inside_soil(px, py)) {
                double d6[2][3];
                planewave(wave, time - t0, px - prob->worigin[0], py - prob->worigin[1], d6);
                fx = fx + d6[0][0];
                fy = fy + d6[1][0];
            }
            out[(size_t)save * nrecv * 2 + 2 * i] = fx;
            out[(size_t)save * nrecv * 2 + 2 * i + 1] = fy;
        }
    }
};

}  // namespace

extern "C" {

const char *oracle_last_error(void) { return g_err.c_str(); }

void oracle_calck(double m, double l, double *k64) { calck(m, l, k64); }
void oracle_calcsqm(double *m64) { calcsqm(m64); }

void oracle_multdrm(const double *k64, const double *u8, const unsigned char *e8, double *p8) {
    bool e[8];
    for (int i = 0; i < 8; ++i) e[i] = e8[i] != 0;
    multdrm(k64, u8, e, p8);
}

// Free field at (t, x1, x3) for one wave: u6 = [ux, uz, vx, vz, ax, az].
int oracle_planewave(int kind, double amp, double alpha, double beta, double angle, double freq, double t,
                     double x1, double x3, double *u6) {
    PWave w;
    int rc = initplanewaves(w, kind, amp, alpha, beta, angle, freq);
    if (rc) return rc;
    double u[2][3];
    planewave(w, t, x1, x3, u);
    for (int c = 0; c < 3; ++c) { u6[2 * c] = u[0][c]; u6[2 * c + 1] = u[1][c]; }
    return 0;
}

// Run init_explicit + run_explicit for one right-hand side.
//   rhs        0-based index into prob->waves
//   hang_mode  EXFEM_HANG_HALF or EXFEM_HANG_LITERAL
//   nthreads   1 = the reference's sequential loop; >1 = element terms in
//              parallel, summed per dof in element order (bit-identical)
//   nsteps     steps to run (<= prob->nsteps)
// Outputs (each may be NULL): mfull_out[2*nnodes] (mass.bin content),
// seis_out[(nsteps/io_interval+1)*nrecv*2], u_out[2*nnodes], seconds_out
// (wall time of the stepping loop only).
int oracle_run(const exfem_mesh *mesh, const exfem_problem *prob, int rhs, int hang_mode, int nthreads,
               int nsteps, double *mfull_out, double *seis_out, double *u_out, double *seconds_out) {
    if (!mesh || !prob || rhs < 0 || rhs >= prob->nrhs || nsteps < 0) { g_err = "bad arguments"; return EXFEM_E_ARG; }
    Solver S;
    S.mesh = mesh;
    S.prob = prob;
    S.nn = mesh->nnodes;
    S.ne = mesh->nelems;
    S.hang_mode = hang_mode;
    S.dt = prob->deltat;
    // setupconstants (explicit.f90:72-77)
    S.ea[0] = 1.0 / (S.dt * S.dt);
    S.ea[1] = 1.0 / (2.0 * S.dt);
    S.ea[2] = 2.0 * S.ea[0];
    S.ea[3] = 1.0 / S.ea[1];
    // problem_setup: calcsqm, init_stiffness (model.f90:958-962, 1099-1106)
    calcsqm(S.mmat);
    S.kmat.resize((size_t)64 * prob->nmat);
    for (int i = 0; i < prob->nmat; ++i) calck(prob->matconst[5 * i], prob->matconst[5 * i + 1], &S.kmat[(size_t)64 * i]);
    for (int e = 0; e < S.ne; ++e) {
        int cnt = 0;
        for (int j = mesh->eptr[e] - 1; j < mesh->eptr[e + 1] - 1; ++j) cnt += !mesh->ediv[j];
        if (cnt != 4) { g_err = "element " + std::to_string(e + 1) + " has " + std::to_string(cnt) + " non-hanging nodes"; return EXFEM_E_MESH; }
    }
    if (prob->waves) {
        const exfem_wave &wv = prob->waves[rhs];
        int rc = initplanewaves(S.wave, wv.kind, wv.amp, prob->walpha, prob->wbeta, wv.angle, wv.freq);
        if (rc) return rc;
        S.t0 = wv.t0;
    } else if (prob->nseismic > 0) {
        g_err = "a DRM layer needs waves";
        return EXFEM_E_ARG;
    } else {
        S.have_wave = false;
    }
    const int ndof = 2 * S.nn;
    // setup_point_source (model.f90:1051-1078): unique point nodes
    const int pkind = prob->point_kind;
    if (pkind != 0) {
        std::vector<char> flag(S.nn, 0);
        for (int i = 0; i < prob->npoint; ++i) {
            int g = prob->point_nodes[i];
            if (g < 1 || g > S.nn) { g_err = "point source node out of range"; return EXFEM_E_ARG; }
            flag[g - 1] = 1;
        }
        for (int n = 0; n < S.nn; ++n)
            if (flag[n]) S.pdofs.push_back(2 * n + 1);
    }
    const double pamp = prob->point_amp, psig = prob->point_sigma, pt0 = prob->point_t0;
    // init_explicit (explicit.f90:79-109)
    S.u.assign(ndof, 0.0);
    S.up.assign(ndof, 0.0);
    if (pkind == EXFEM_POINT_DISP) {   // problem_displacements at 0 and -dt (explicit.f90:93-94)
        for (int d : S.pdofs) S.u[d] = ricker_point(pamp, psig, 0.0 - pt0);
        for (int d : S.pdofs) S.up[d] = ricker_point(pamp, psig, -S.dt - pt0);
    }
    S.mfull.assign(ndof, 0.0);
    S.ro.assign(ndof, 0.0);
    for (int i = 0; i < S.ne; ++i) {
        int dofs[8];
        S.elemallnhdofs(i, dofs);
        double mass = S.getmassof(i), damping[8];
        S.getdampingof(i, damping);
        // explicit.f90:100-102 adds left to right: (e_mfull + e_a(2)*damping) + e_a(1)*mass
        for (int k = 0; k < 8; ++k) S.mfull[dofs[k] - 1] = (S.mfull[dofs[k] - 1] + S.ea[1] * damping[k]) + S.ea[0] * mass;
    }
    S.sum_reactanchors(S.mfull);
    if (mfull_out) std::memcpy(mfull_out, S.mfull.data(), sizeof(double) * ndof);

    const int nrecv = prob->nrecv;
    const int io = prob->io_interval > 0 ? prob->io_interval : 1;
    std::vector<double> seis;
    if (seis_out) seis.assign((size_t)(nsteps / io + 1) * nrecv * 2, 0.0);
    if (seis_out) S.sample(0, seis, nrecv);

    // parallel element pass: per-dof contribution lists in element order
    std::vector<int> cptr, clist;
    std::vector<double> ebuf;
    if (nthreads > 1) {
        cptr.assign(ndof + 1, 0);
        for (int e = 0; e < S.ne; ++e) {
            int dofs[8];
            S.elemallnhdofs(e, dofs);
            for (int k = 0; k < 8; ++k) cptr[dofs[k]]++;
        }
        for (int d = 0; d < ndof; ++d) cptr[d + 1] += cptr[d];
        clist.resize(cptr[ndof]);
        std::vector<int> fill(cptr.begin(), cptr.end() - 1);
        for (int e = 0; e < S.ne; ++e) {
            int dofs[8];
            S.elemallnhdofs(e, dofs);
            for (int k = 0; k < 8; ++k) clist[fill[dofs[k] - 1]++] = e * 8 + k;
        }
        ebuf.resize((size_t)S.ne * 8);
    }
#ifdef _OPENMP
    if (nthreads > 1) omp_set_num_threads(nthreads);
#endif
    auto t_start = std::chrono::steady_clock::now();
    for (int i = 1; i <= nsteps; ++i) {
        std::fill(S.ro.begin(), S.ro.end(), 0.0);
        S.wave_reactions((double)i * S.dt, S.ro);   // additive_reactions (explicit.f90:128)
        if (nthreads <= 1) {
            for (int j = 0; j < S.ne; ++j) {
                double localr[8];
                int dofs[8];
                S.element_term(j, localr, dofs);
                for (int k = 0; k < 8; ++k) S.ro[dofs[k] - 1] = S.ro[dofs[k] - 1] + localr[k];
            }
        } else {
#pragma omp parallel for schedule(static)
            for (int j = 0; j < S.ne; ++j) {
                int dofs[8];
                S.element_term(j, &ebuf[(size_t)j * 8], dofs);
            }
#pragma omp parallel for schedule(static)
            for (int d = 0; d < ndof; ++d) {
                double acc = S.ro[d];
                for (int q = cptr[d]; q < cptr[d + 1]; ++q) acc = acc + ebuf[clist[q]];
                S.ro[d] = acc;
            }
        }
        if (pkind == EXFEM_POINT_FORCE)              // absolute_reactions (explicit.f90:144)
            for (int d : S.pdofs) S.ro[d] = S.ro[d] + ricker_point(pamp, psig, (double)i * S.dt - pt0);
        S.sum_reactanchors(S.ro);                    // explicit.f90:145
        S.up.swap(S.u);                              // e_up = e_u (147)
        for (int d = 0; d < ndof; ++d) S.u[d] = S.ro[d] / S.mfull[d];   // (148)
        if (pkind == EXFEM_POINT_DISP)               // problem_displacements (explicit.f90:150)
            for (int d : S.pdofs) S.u[d] = ricker_point(pamp, psig, (double)i * S.dt - pt0);
        S.set_dispshanging(S.u);                     // (151)
        if (seis_out && i % io == 0) S.sample(i / io, seis, nrecv);
        if (!std::isfinite(S.u[0])) { /* keep going: callers inspect the output */ }
    }
    auto t_end = std::chrono::steady_clock::now();
    if (seconds_out) *seconds_out = std::chrono::duration<double>(t_end - t_start).count();
    if (seis_out) std::memcpy(seis_out, seis.data(), sizeof(double) * seis.size());
    if (u_out) std::memcpy(u_out, S.u.data(), sizeof(double) * ndof);
    return 0;
}

}  // extern "C"
