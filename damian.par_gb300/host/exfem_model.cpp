// exfem_model.cpp — host-side model builder (the Fortran host's role in
// damian.par): problem.in parsing, materials, single-process quadtree mesher,
// problem setup, time-step selection and receiver search.  Everything here is
// FP64 and runs once per problem; the time loop lives in the CUDA library.
//
// Reference map (file:line in damian.par):
//   parse              io.cpp:113-228 (load_problem_file)
//   materials          model.f90:893-945, formulation.f90:62-217
//   problem params     model.f90:856-889, formulation.f90:20-31
//   DRM box / wave     model.f90:982-1001, 197-241
//   mesher             mesh_utils.f90:64-112 (initial_mesh), 720-750 (cut_geom),
//                      454-681 (final_division); divide selection
//                      mesh_utils.f90:114-201 with communicator.f90:627-768;
//                      node creation mesh_utils.f90:203-409
//   division tests     model.f90:252-445 (needs_division/needs_deletion/material_prop)
//   problem_setup      model.f90:958-1106 (hanging, absorbing, wave_elems)
//   time step          communicator.f90:1629-1662 (recalculate_deltat)
//   receivers          visualization.f90:286-305, quadtree.f90:253-291
#include "exfem_host.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <random>
#include <sstream>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

// Tolerance compares of utilities.f90:159-175 (u_tol = 1e-9, utilities.f90:8).
constexpr double U_TOL = 1.0e-9;
inline bool realequal(double a, double b) { return std::fabs(a - b) < U_TOL; }
inline bool realunder(double a, double b) { return (a - b) < -U_TOL; }
inline bool realover(double a, double b) { return (a - b) > U_TOL; }

// ---------------------------------------------------------------- deck ----
struct Deck {
    double width = 0, height = 0, time = 0, inttime = 0, chper = 0;
    double nperlen = 0, sperlen = 0;
    bool have_control = false, have_domain = false, have_time = false, have_chper = false;
    int nmats = 0;
    std::vector<char> cmats;     // 2*nmats
    std::vector<double> vmats;   // 3*nmats
    std::string prob = "      ", geom = "NONE  ";
    std::vector<double> pparams, gparams;
    // extensions
    bool have_recv = false;
    double rxmin = 0, rxmax = 0, rdist = 1;
    std::vector<exfem_wave> rhs;
    bool have_rhs = false;
    int refine_levels = 0;
    double refine_band = 0;
    double het_sigma = 0;
    unsigned long long het_seed = 0;
};

std::string fixed6(const std::string &line) {
    std::string s(6, ' ');
    for (size_t i = 0; i < 6 && i < line.size(); ++i) s[i] = line[i];
    return s;
}

int parse_deck(const char *text, Deck &d) {
    std::istringstream in(text ? text : "");
    std::string line, section;
    auto next = [&](std::string &out) -> bool {
        if (!std::getline(in, out)) return false;
        if (!out.empty() && out.back() == '\r') out.pop_back();
        return true;
    };
    if (!next(line) || line != "PROBLEM FILE EXFEM")
        return fail(EXFEM_E_ARG, "deck: first line must be 'PROBLEM FILE EXFEM'");
    while (next(section)) {
        if (section == "DOMAIN:") {
            if (!next(line)) break;
            std::istringstream is(line);
            is >> d.width >> d.height;
            d.have_domain = true;
        } else if (section == "CH PERIOD:") {
            if (!next(line)) break;
            std::istringstream is(line);
            is >> d.chper;
            d.have_chper = true;
        } else if (section == "TIME:") {
            if (!next(line)) break;
            std::istringstream is(line);
            is >> d.time >> d.inttime;
            d.have_time = true;
        } else if (section == "CONTROL:") {
            if (!next(line)) break;
            std::istringstream is(line);
            is >> d.nperlen >> d.sperlen;
            d.have_control = true;
        } else if (section == "MATERIALS:") {
            if (!next(line)) break;
            std::istringstream is(line);
            is >> d.nmats;
            if (d.nmats <= 0 || d.nmats > 1000000) return fail(EXFEM_E_ARG, "deck: bad material count");
            d.cmats.assign(2 * d.nmats, ' ');
            d.vmats.assign(3 * d.nmats, 0.0);
            for (int i = 0; i < d.nmats; ++i) {
                if (!next(line)) return fail(EXFEM_E_ARG, "deck: truncated MATERIALS");
                std::istringstream iss(line);
                std::string s;
                iss >> s; d.cmats[2 * i] = s.empty() ? ' ' : s[0];
                iss >> d.vmats[3 * i];
                iss >> s; d.cmats[2 * i + 1] = s.empty() ? ' ' : s[0];
                iss >> d.vmats[3 * i + 1] >> d.vmats[3 * i + 2];
            }
        } else if (section == "PROBLEM:") {
            if (!next(line)) break;
            d.prob = fixed6(line);
            if (!next(line)) break;
            std::istringstream is(line);
            int n = 0;
            is >> n;
            d.pparams.assign(std::max(n, 0), 0.0);
            for (int i = 0; i < n; ++i) is >> d.pparams[i];
        } else if (section == "GEOMETRY:") {
            if (!next(line)) break;
            d.geom = fixed6(line);
            if (!next(line)) break;
            std::istringstream is(line);
            int n = 0;
            is >> n;
            d.gparams.assign(std::max(n, 0), 0.0);
            for (int i = 0; i < n; ++i) is >> d.gparams[i];
        } else if (section == "RECEIVERS:") {
            if (!next(line)) break;
            std::istringstream is(line);
            is >> d.rxmin >> d.rxmax >> d.rdist;
            d.have_recv = true;
        } else if (section == "RHS:") {
            if (!next(line)) break;
            std::istringstream is(line);
            int n = 0;
            is >> n;
            if (n <= 0 || n > 4096) return fail(EXFEM_E_ARG, "deck: bad RHS count");
            d.rhs.clear();
            for (int i = 0; i < n; ++i) {
                if (!next(line)) return fail(EXFEM_E_ARG, "deck: truncated RHS");
                std::istringstream iss(line);
                std::string kind;
                exfem_wave w{};
                iss >> kind >> w.angle >> w.amp >> w.freq >> w.t0;
                if (kind == "WAVEP") w.kind = EXFEM_WAVE_P;
                else if (kind == "WAVESV") w.kind = EXFEM_WAVE_SV;
                else return fail(EXFEM_E_ARG, "deck: RHS kind must be WAVEP or WAVESV");
                d.rhs.push_back(w);
            }
            d.have_rhs = true;
        } else if (section == "REFINE:") {
            if (!next(line)) break;
            std::istringstream is(line);
            is >> d.refine_levels >> d.refine_band;
        } else if (section == "HETEROGENEITY:") {
            if (!next(line)) break;
            std::istringstream is(line);
            is >> d.het_sigma >> d.het_seed;
        }
    }
    if (!d.have_domain || !d.have_time || !d.have_chper || !d.have_control || d.nmats <= 0)
        return fail(EXFEM_E_ARG, "deck: DOMAIN:, TIME:, CH PERIOD:, CONTROL: and MATERIALS: are required");
    if (d.nperlen <= 0 || d.sperlen <= 0) return fail(EXFEM_E_ARG, "deck: CONTROL values must be positive");
    return 0;
}

// ----------------------------------------------- material conversions ----
// formulation.f90:5-11 parameter ids.
enum { F_YOUNG = 1, F_NU = 2, F_SHEAR = 3, F_BULK = 4, F_LAMBDA = 5, F_VP = 1, F_VS = 2 };

int c_to_p(char c) {  // formulation.f90:100-118
    switch (c) {
        case 'E': return F_YOUNG;
        case 'v': return F_NU;
        case 'G': return F_SHEAR;
        case 'K': return F_BULK;
        case 'l': return F_LAMBDA;
        default: return 0;
    }
}
int c_to_v(char c) {  // formulation.f90:120-132
    if (c == 'p') return F_VP;
    if (c == 's') return F_VS;
    return 0;
}

// e_to_e (formulation.f90:135-217): fill in the remaining elastic constants
// from the two given, iterating the closed-form relations.
bool e_to_e(const int pfrom[2], const double param[2], int nto, const int *pto, double *res) {
    double from[6] = {0, 0, 0, 0, 0, 0};
    bool found[6] = {false, false, false, false, false, false};
    for (int i = 0; i < 2; ++i) { from[pfrom[i]] = param[i]; found[pfrom[i]] = true; }
    auto all_found = [&]() { for (int k = 0; k < nto; ++k) if (!found[pto[k]]) return false; return true; };
    for (int it = 0; it < 3; ++it) {
        if (all_found()) break;
        for (int j = 1; j <= 5; ++j) {
            if (found[j]) continue;
            switch (j) {
                case F_YOUNG:
                    if (found[F_SHEAR] && found[F_NU]) { found[F_YOUNG] = true; from[F_YOUNG] = 2 * (1 + from[F_NU]) * from[F_SHEAR]; }
                    else if (found[F_BULK] && found[F_NU]) { found[F_YOUNG] = true; from[F_YOUNG] = 3 * (1 - 2 * from[F_NU]) * from[F_BULK]; }
                    else if (found[F_LAMBDA] && found[F_NU]) {
                        found[F_YOUNG] = true;
                        from[F_YOUNG] = (1 - 2 * from[F_NU]) * (1 + from[F_NU]);
                        from[F_YOUNG] = from[F_YOUNG] * from[F_LAMBDA] / from[F_NU];
                    }
                    break;
                case F_NU:
                    if (found[F_YOUNG] && found[F_SHEAR]) { found[F_NU] = true; from[F_NU] = (from[F_YOUNG] - 2 * from[F_SHEAR]) / (2 * from[F_SHEAR]); }
                    else if (found[F_YOUNG] && found[F_BULK]) { found[F_NU] = true; from[F_NU] = (3 * from[F_BULK] - from[F_YOUNG]) / (6 * from[F_BULK]); }
                    else if (found[F_BULK] && found[F_SHEAR]) { found[F_NU] = true; from[F_NU] = (3 * from[F_BULK] - 2 * from[F_SHEAR]) / (6 * from[F_BULK] + 2 * from[F_SHEAR]); }
                    else if (found[F_SHEAR] && found[F_LAMBDA]) { found[F_NU] = true; from[F_NU] = from[F_LAMBDA] / (2 * (from[F_LAMBDA] + from[F_SHEAR])); }
                    else if (found[F_BULK] && found[F_LAMBDA]) { found[F_NU] = true; from[F_NU] = from[F_LAMBDA] / (3 * from[F_BULK] - from[F_LAMBDA]); }
                    break;
                case F_SHEAR:
                    if (found[F_YOUNG] && found[F_NU]) { found[F_SHEAR] = true; from[F_SHEAR] = from[F_YOUNG] / (2 * (from[F_NU] + 1)); }
                    break;
                case F_BULK:
                    if (found[F_YOUNG] && found[F_NU]) { found[F_BULK] = true; from[F_BULK] = from[F_YOUNG] / (3 * (1 - 2 * from[F_NU])); }
                    break;
                case F_LAMBDA:
                    if (found[F_YOUNG] && found[F_NU]) {
                        found[F_LAMBDA] = true;
                        from[F_LAMBDA] = from[F_YOUNG] * from[F_NU] / ((1 + from[F_NU]) * (1 - 2 * from[F_NU]));
                    }
                    break;
            }
        }
    }
    if (!all_found()) return false;
    for (int k = 0; k < nto; ++k) res[k] = from[pto[k]];
    return true;
}

// v_to_e (formulation.f90:62-71) into (mu, lambda).
void v_to_lame(double vp, double vs, double rho, double *mu, double *lambda) {
    double l1 = rho * vs * vs;
    double l2 = rho * vp * vp - 2 * l1;
    *mu = l1;
    *lambda = l2;
}

// setup_materials (model.f90:893-945): m_matconst(5, nmat) = (mu, lambda, rho, vp, vs).
int setup_materials(Deck &d, std::vector<double> &mc) {
    mc.assign(5 * d.nmats, 0.0);
    for (int i = 0; i < d.nmats; ++i) {
        char *cm = &d.cmats[2 * i];
        double *vm = &d.vmats[3 * i];
        double *m = &mc[5 * i];
        int im[2] = {c_to_p(cm[0]), c_to_p(cm[1])};
        if (im[0] == 0 || im[1] == 0) {
            if (im[1] == F_NU) {
                std::swap(im[0], im[1]); std::swap(cm[0], cm[1]); std::swap(vm[0], vm[1]);
            }
            if (im[0] == F_NU) {
                im[1] = c_to_v(cm[1]);
                if (im[1] == 0) return fail(EXFEM_E_ARG, "Not recognized material");
                // v_nu_to_v (formulation.f90:85-97)
                double nu = vm[0], vin = vm[1];
                double rel = std::sqrt(2.0 * (nu - 1.0) / (2.0 * nu - 1.0));
                double v[3] = {0, 0, 0};
                v[im[1]] = vin;
                if (im[1] == F_VS) v[F_VP] = rel * v[F_VS];
                else v[F_VS] = v[F_VP] / rel;
                m[3] = v[F_VP]; m[4] = v[F_VS];
                m[2] = vm[2];
                v_to_lame(m[3], m[4], m[2], &m[0], &m[1]);
            } else if (im[0] == 0 && im[1] == 0) {
                im[0] = c_to_v(cm[0]); im[1] = c_to_v(cm[1]);
                if (im[0] == 0 || im[1] == 0) return fail(EXFEM_E_ARG, "Not recognized material");
                m[2 + im[0]] = vm[0];
                m[2 + im[1]] = vm[1];
                m[2] = vm[2];
                v_to_lame(m[3], m[4], m[2], &m[0], &m[1]);
            } else {
                return fail(EXFEM_E_ARG, "Not recognized material");
            }
        } else {
            const int pto[2] = {F_SHEAR, F_LAMBDA};
            double lame[2];
            if (!e_to_e(im, vm, 2, pto, lame)) return fail(EXFEM_E_ARG, "Conversion not valid");
            m[0] = lame[0]; m[1] = lame[1]; m[2] = vm[2];
            // e_to_v (formulation.f90:74-83)
            m[3] = std::sqrt((m[1] + 2 * m[0]) / m[2]);
            m[4] = std::sqrt(m[0] / m[2]);
        }
        if (!(m[2] > 0) || !(m[3] > 0) || !(m[4] > 0) || !std::isfinite(m[0]) || !std::isfinite(m[1]))
            return fail(EXFEM_E_ARG, "material " + std::to_string(i + 1) + " has non-positive rho/vp/vs");
    }
    return 0;
}

// --------------------------------------------------------------- model ----
struct Model {
    Deck deck;
    int nmat_base = 0;
    std::vector<double> matconst;     // 5*nmat
    std::vector<double> probconst;    // 2*nmat_base: (length, step)
    double blength = 0, mlength = 0, duration = 0, deltat = 0, inttime = 0;
    int nsteps = 0, nsteps_deck = 0, totcols = 0, totrows = 0, io_interval = 1;
    bool is_wave = false;
    int wrows = 0, wcols = 0, wzero = 0;
    double worigin[2] = {0, 0};
    double walpha = 0, wbeta = 0;
    double wleft = 0, wright = 0, wtop = 0;
    // mesh (0-based internally)
    std::vector<int> eptr{0};
    std::vector<int> eind;
    std::vector<uint8_t> ediv;
    std::vector<int> emat;            // 1-based material ids
    std::vector<double> nx, ny;
    // problem (1-based for export)
    std::vector<int> absorbing, hanging, seismic;
    std::vector<double> recv_xy;
    std::vector<int> recv_elem;
    std::vector<exfem_wave> waves;
    // point source (setup_point_source): kind, Ricker parameters, 1-based nodes
    int point_kind = 0;
    double point_amp = 0, point_sigma = 0, point_t0 = 0, point_dist = 0;
    std::vector<int> point_nodes;
    // exported 1-based mesh arrays
    std::vector<int> x_eptr, x_eind;
    std::vector<double> x_nodes;
    int nlevels = 1;
    double min_h = 0, max_h = 0;

    int ne() const { return (int)eptr.size() - 1; }

    // elemallnhnodes (model.f90:163-174): the four non-hanging corners.
    bool corners(int e, int c[4]) const {
        int k = 0;
        for (int j = eptr[e]; j < eptr[e + 1]; ++j)
            if (!ediv[j]) { if (k < 4) c[k] = eind[j]; ++k; }
        return k == 4;
    }
    // elength (model.f90:112-118)
    double elength(int e) const {
        int c[4];
        corners(e, c);
        return ny[c[2]] - ny[c[0]];
    }

    // setup_point_source (model.f90:1051-1078): every node closer than the
    // distance to one of the points (distance, utilities.f90:210-214), unique
    // and in node order.
    void setup_point_source() {
        if (!point_kind) return;
        const std::vector<double> &pp = deck.pparams;
        std::vector<char> hit(nx.size(), 0);
        for (size_t j = 4; j + 1 < pp.size(); j += 2)
            for (size_t i = 0; i < nx.size(); ++i) {
                double dx = pp[j] - nx[i], dy = pp[j + 1] - ny[i];
                if (std::sqrt(dx * dx + dy * dy) < point_dist) hit[i] = 1;
            }
        point_nodes.clear();
        for (size_t i = 0; i < nx.size(); ++i)
            if (hit[i]) point_nodes.push_back((int)i + 1);
    }

    // inside_soil (model.f90:217-235): outside the DRM box
    bool inside_soil(double x, double y) const {
        if (!is_wave) return false;
        return realunder(x, wleft) || realover(x, wright) || realover(y, wtop);
    }
    bool void_soil(double, double y) const { return realunder(y, worigin[1]); }  // model.f90:237-241

    // material_prop (model.f90:397-445) + EVALLY
    int material_prop(double x, double y) const {
        if (inside_soil(x, y)) return (int)deck.pparams[4];
        const std::string &g = deck.geom;
        const std::vector<double> &gp = deck.gparams;
        if (g == "VALLEY" && gp.size() >= 3) {
            double d = std::sqrt((x - gp[0]) * (x - gp[0]) + (y - gp[1]) * (y - gp[1]));
            return d < gp[2] ? 2 : 1;
        }
        if (g == "VARECT" && gp.size() >= 4) {
            return (std::fabs(x - gp[0]) < gp[2] && std::fabs(y - gp[1]) < gp[3]) ? 2 : 1;
        }
        if (g == "EVALLY" && gp.size() >= 4) {
            double dx = (x - gp[0]) / gp[2], dy = (y - gp[1]) / gp[3];
            return (dx * dx + dy * dy) < 1.0 ? 2 : 1;
        }
        return 1;
    }

    // Geometric refinement band (REFINE: extension): true when the point lies
    // within `band` (+ half a diagonal of the element) of the canyon rim or of
    // the valley boundary.
    bool near_feature(double x, double y, double elen) const {
        const std::string &g = deck.geom;
        const std::vector<double> &gp = deck.gparams;
        double band = deck.refine_band + 0.7072 * elen;
        if ((g == "CANYON" || g == "VALLEY") && gp.size() >= 3) {
            double d = std::sqrt((x - gp[0]) * (x - gp[0]) + (y - gp[1]) * (y - gp[1]));
            return std::fabs(d - gp[2]) < band;
        }
        if (g == "EVALLY" && gp.size() >= 4) {
            double dx = (x - gp[0]) / gp[2], dy = (y - gp[1]) / gp[3];
            double s = std::sqrt(dx * dx + dy * dy);
            return std::fabs(s - 1.0) * std::min(gp[2], gp[3]) < band;
        }
        return false;
    }

    // needs_division (model.f90:252-292) with the REFINE: extension.
    bool needs_division(int e) const {
        double elen = elength(e);
        if (realover(elen, mlength)) return false;
        int c[4];
        corners(e, c);
        double cx = (nx[c[0]] + nx[c[1]] + nx[c[2]] + nx[c[3]]) / 4.0;
        double cy = (ny[c[0]] + ny[c[1]] + ny[c[2]] + ny[c[3]]) / 4.0;
        if (deck.refine_levels > 0) {
            double minlen = blength / std::ldexp(1.0, deck.refine_levels);
            if (realover(elen, minlen) && !inside_soil(cx, cy) && near_feature(cx, cy, elen)) return true;
        }
        int mat = material_prop(cx, cy);
        double leng = probconst[2 * (mat - 1)];
        if (leng < elen) return true;
        if (inside_soil(cx, cy)) return false;
        leng = std::numeric_limits<double>::infinity();
        for (int i = -1; i <= 1; i += 2) {
            int m1 = material_prop(cx + i * elen, cy);
            leng = std::min(leng, probconst[2 * (m1 - 1)]);
            int m2 = material_prop(cx, cy + i * elen);
            leng = std::min(leng, probconst[2 * (m2 - 1)]);
        }
        return (leng * 2.0) < elen;
    }

    // needs_deletion (model.f90:303-388) for the NONE/CANYON/RECTAN geometries.
    bool needs_deletion(int e) const {
        int c[4];
        corners(e, c);
        double elen = elength(e);
        if (realover(elen, mlength)) return false;
        double px = (nx[c[0]] + nx[c[1]] + nx[c[2]] + nx[c[3]]) / 4.0;
        double py = (ny[c[0]] + ny[c[1]] + ny[c[2]] + ny[c[3]]) / 4.0;
        if (inside_soil(px, py)) return void_soil(px, py);
        const std::string &g = deck.geom;
        const std::vector<double> &gp = deck.gparams;
        if (g == "CANYON" && gp.size() >= 3) {
            for (int i = 0; i < 4; ++i) {
                double dx = nx[c[i]] - gp[0], dy = ny[c[i]] - gp[1];
                if (std::sqrt(dx * dx + dy * dy) > gp[2]) return false;
            }
            return true;
        }
        if (g == "RECTAN" && gp.size() >= 4) {
            for (int i = 0; i < 4; ++i)
                if (std::fabs(nx[c[i]] - gp[0]) > gp[2] || std::fabs(ny[c[i]] - gp[1]) > gp[3]) return false;
            return true;
        }
        return false;
    }

    int setup_problem_params();
    void init_wave();
    void initial_mesh();
    void cut_geom();
    bool divide_pass();
    void setup_hanging();
    void create_absorbingbc();
    void wave_elems();
    void apply_heterogeneity();
    void recalculate_deltat();
    int find_receivers();
    void export_arrays();
};

// setup_problem_params (model.f90:856-889)
int Model::setup_problem_params() {
    int nm = nmat_base;
    probconst.assign(2 * nm, 0.0);
    double length = 0.0, dt = std::numeric_limits<double>::infinity();
    for (int i = 0; i < nm; ++i) {
        // explicitparams (formulation.f90:20-25)
        double alpha = matconst[5 * i + 3], beta = matconst[5 * i + 4];
        double l = (deck.chper * beta) / deck.nperlen;
        double s = (l / alpha) / deck.sperlen;
        probconst[2 * i] = l;
        probconst[2 * i + 1] = s;
        if (length < l) length = l;
        if (dt > s) dt = s;
    }
    if (!(length > 0)) return fail(EXFEM_E_ARG, "non-positive characteristic length");
    int m = (int)std::ceil(deck.height / length);
    length = deck.height / (double)m;
    int n = (int)std::ceil(deck.width / length);
    int steps = (int)std::ceil(deck.time / dt);
    if (steps <= 0) return fail(EXFEM_E_ARG, "TIME: duration must be positive");
    dt = deck.time / (double)steps;
    duration = dt * steps;
    blength = length;
    mlength = blength;
    totcols = n + 1;
    totrows = m + 1;
    nsteps = steps;
    deltat = dt;
    if ((double)totcols * (double)totrows > 4.0e8) return fail(EXFEM_E_ARG, "base grid too large");
    return 0;
}

// init_wave (model.f90:982-1001); the box edges are those of inside_soil.
void Model::init_wave() {
    const std::vector<double> &pp = deck.pparams;
    wrows = (int)std::ceil(pp[1] / blength) + 1;
    wcols = (totcols - (1 + (int)std::ceil(pp[0] / blength))) / 2;
    worigin[0] = pp[2];
    worigin[1] = pp[3];
    int mat = (int)pp[4];
    walpha = matconst[5 * (mat - 1) + 3];
    wbeta = matconst[5 * (mat - 1) + 4];
    wzero = (int)std::floor(worigin[1] / blength);
    worigin[1] = (double)wzero * blength;
    wleft = (double)(wcols - 1) * blength;
    wright = (double)((totcols - wcols) - 1) * blength;
    wtop = (double)(wrows - 1) * blength;
}

// initial_mesh (mesh_utils.f90:64-112) on a single rank: nodes column-major
// (x outer, depth inner), element corners (TL, TR, BR, BL) with depth down.
void Model::initial_mesh() {
    int ncols = totcols, nrows = totrows;
    nx.resize((size_t)ncols * nrows);
    ny.resize((size_t)ncols * nrows);
    size_t ind = 0;
    for (int i = 1; i <= ncols; ++i)
        for (int j = 1; j <= nrows; ++j) {
            nx[ind] = (double)(i - 1) * blength;
            ny[ind] = (double)(j - 1) * blength;
            ++ind;
        }
    size_t nel = (size_t)(nrows - 1) * (ncols - 1);
    eptr.assign(1, 0);
    eptr.reserve(nel + 1);
    eind.clear(); eind.reserve(4 * nel);
    ediv.clear(); ediv.reserve(4 * nel);
    emat.clear(); emat.reserve(nel);
    for (int il = 1; il <= ncols - 1; ++il)
        for (int jl = 1; jl <= nrows - 1; ++jl) {
            int a = (il - 1) * nrows + jl, b = il * nrows + jl, c = il * nrows + (jl + 1), d = (il - 1) * nrows + (jl + 1);
            eind.push_back(a - 1); eind.push_back(b - 1); eind.push_back(c - 1); eind.push_back(d - 1);
            for (int k = 0; k < 4; ++k) ediv.push_back(0);
            eptr.push_back((int)eind.size());
            double px = ((double)(il - 1) + 0.5) * blength, py = ((double)(jl - 1) + 0.5) * blength;
            emat.push_back(material_prop(px, py));
        }
}

// cut_geom (mesh_utils.f90:720-750): drop elements that need deletion and the
// nodes nobody references any more, keeping the order of what remains.
void Model::cut_geom() {
    int n = ne();
    std::vector<uint8_t> del(n);
    bool any = false;
    for (int e = 0; e < n; ++e) { del[e] = needs_deletion(e); any = any || del[e]; }
    if (!any) return;
    std::vector<int> neptr{0}, neind;
    std::vector<uint8_t> nediv;
    std::vector<int> nemat;
    neptr.reserve(n + 1); neind.reserve(eind.size()); nediv.reserve(eind.size()); nemat.reserve(n);
    for (int e = 0; e < n; ++e) {
        if (del[e]) continue;
        for (int j = eptr[e]; j < eptr[e + 1]; ++j) { neind.push_back(eind[j]); nediv.push_back(ediv[j]); }
        neptr.push_back((int)neind.size());
        nemat.push_back(emat[e]);
    }
    std::vector<int> remap(nx.size(), -1);
    for (int v : neind) remap[v] = 0;
    int k = 0;
    std::vector<double> nnx, nny;
    for (size_t i = 0; i < nx.size(); ++i)
        if (remap[i] == 0) { remap[i] = k++; nnx.push_back(nx[i]); nny.push_back(ny[i]); }
    for (int &v : neind) v = remap[v];
    eptr.swap(neptr); eind.swap(neind); ediv.swap(nediv); emat.swap(nemat);
    nx.swap(nnx); ny.swap(nny);
}

inline uint64_t pairkey(int a, int b) {
    if (a > b) std::swap(a, b);
    return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b;
}

// One refinement pass: global_divide (communicator.f90:730-768) with the
// selection of mesh_utils.f90:114-201 and the construction of
// mesh_utils.f90:203-409, 454-681, all on a single rank.
bool Model::divide_pass() {
    // One pass of the reference's division (select_local_divide, create_*nodes,
    // select_newhanging, final_division; mesh_utils.f90:114-681).  New nodes are
    // numbered in the reference's order: edge nodes of divided elements with a
    // larger neighbour, then those under an undivided smaller neighbour, then
    // centres, then edges without a neighbour, each in element order.  Every
    // phase counts per element, takes a prefix sum and fills in parallel, so
    // the numbering is the sequential one.
    const int n = ne();
    const int nn = (int)nx.size();
    // node -> element incidence over full CSR (hanging slots included)
    std::vector<int> nptr(nn + 1, 0);
    for (int v : eind) nptr[v + 1]++;
    for (int i = 0; i < nn; ++i) nptr[i + 1] += nptr[i];
    std::vector<int> nel(nptr[nn]);
    {
        std::vector<int> fill(nptr.begin(), nptr.end() - 1);
        for (int e = 0; e < n; ++e)
            for (int j = eptr[e]; j < eptr[e + 1]; ++j) nel[fill[eind[j]]++] = e;
    }
    // dual graph with ncommon = 2 (parmetis_v3_mesh2dual, communicator.f90:496-514),
    // each element's neighbours in ascending order
    constexpr int MAXN = 16;
    std::vector<int> nbuf((size_t)n * MAXN), deg(n, 0);
    int overflow = 0;
#pragma omp parallel for schedule(static) reduction(| : overflow)
    for (int e = 0; e < n; ++e) {
        int cand[128];
        int nc = 0;
        for (int j = eptr[e]; j < eptr[e + 1]; ++j) {
            const int v = eind[j];
            for (int q = nptr[v]; q < nptr[v + 1]; ++q)
                if (nel[q] != e && nc < 128) cand[nc++] = nel[q];
        }
        std::sort(cand, cand + nc);
        int d = 0;
        for (int i = 0; i < nc;) {
            int k = i + 1;
            while (k < nc && cand[k] == cand[i]) ++k;
            if (k - i >= 2) {
                if (d < MAXN) nbuf[(size_t)e * MAXN + d] = cand[i];
                ++d;
            }
            i = k;
        }
        if (d > MAXN || nc >= 128) overflow = 1;
        deg[e] = std::min(d, MAXN);
    }
    if (overflow) {   // cannot happen on a 2:1 quadtree; keep the mesh as it is
        return false;
    }
    std::vector<int> aptr(n + 1, 0);
    for (int e = 0; e < n; ++e) aptr[e + 1] = aptr[e] + deg[e];
    std::vector<int> adj(aptr[n]);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < n; ++e)
        for (int d = 0; d < deg[e]; ++d) adj[aptr[e] + d] = nbuf[(size_t)e * MAXN + d];
    std::vector<int>().swap(nbuf);
    auto hanging_element = [&](int e) { return (eptr[e + 1] - eptr[e]) > 4; };   // model.f90:454-458
    // select_local_divide (mesh_utils.f90:114-154)
    std::vector<uint8_t> todiv(n, 0);
    int further = 0;
#pragma omp parallel for schedule(static) reduction(| : further)
    for (int e = 0; e < n; ++e) {
        if (needs_division(e) && !hanging_element(e)) {
            bool ok = true;
            for (int q = aptr[e]; q < aptr[e + 1]; ++q)
                if (hanging_element(adj[q])) { ok = false; break; }
            todiv[e] = ok;
            further |= ok ? 1 : 0;
        }
    }
    if (!further) return false;
    mlength = mlength / 2.0;

    // edge_connects (model.f90:494-516): edge index (0-based) of e shared with f
    auto edge_of = [&](int e, int f) -> int {
        int sa = eptr[e + 1] - eptr[e], sb = eptr[f + 1] - eptr[f];
        const int *A = &eind[eptr[e]], *B = &eind[eptr[f]];
        for (int ia = 0; ia < sa; ++ia)
            for (int ib = 0; ib < sb; ++ib) {
                int na = (ia + 1) % sa, nb = (ib + 1) % sb;
                if (A[ia] == B[nb] && A[na] == B[ib]) return ia;
            }
        return -1;
    };
    auto midpoint = [&](int e, int j, double &px, double &py) {  // elementnodes(e, j, 2)
        int s = eptr[e + 1] - eptr[e];
        int a = eind[eptr[e] + j], b = eind[eptr[e] + (j + 1) % s];
        px = (nx[a] + nx[b]) / 2.0;
        py = (ny[a] + ny[b]) / 2.0;
    };
    // the slot of i in k's neighbour list
    auto slot_of = [&](int k, int i) -> int {
        for (int q = aptr[k]; q < aptr[k + 1]; ++q)
            if (adj[q] == i) return q;
        return -1;
    };
    // adjnode[q]: the node created on the edge between element e and adj[q]
    // (both slots of the pair carry it), -1 if none
    std::vector<int> adjnode(aptr[n], -1);
    std::vector<int> cnt(n + 1, 0);
    const int base = nn;
    int next = base;
    auto scan = [&]() {   // cnt[1..n] -> exclusive offsets starting at next
        int acc = next;
        for (int i = 0; i < n; ++i) { int c = cnt[i + 1]; cnt[i + 1] = acc; acc += c; }
        next = acc;
    };
    std::vector<double> addx, addy;
    auto grow = [&](int upto) { addx.resize(upto - base); addy.resize(upto - base); };
    // create_edgenodes: over edges (todivide element, larger neighbour)
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        int c = 0;
        if (todiv[i])
            for (int q = aptr[i]; q < aptr[i + 1]; ++q)
                if (i < adj[q] && edge_of(i, adj[q]) >= 0) ++c;
        cnt[i + 1] = c;
    }
    scan();
    grow(next);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        if (!todiv[i]) continue;
        int id = cnt[i + 1];
        for (int q = aptr[i]; q < aptr[i + 1]; ++q) {
            int k = adj[q];
            if (!(i < k)) continue;
            int j = edge_of(i, k);
            if (j < 0) continue;
            midpoint(i, j, addx[id - base], addy[id - base]);
            adjnode[q] = id;
            int qk = slot_of(k, i);
            if (qk >= 0) adjnode[qk] = id;
            ++id;
        }
    }
    // ... then under edges whose smaller neighbour is not divided
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k) {
        int c = 0;
        if (todiv[k])
            for (int q = aptr[k]; q < aptr[k + 1]; ++q) {
                int i2 = adj[q];
                if (i2 < k && !todiv[i2] && edge_of(i2, k) >= 0) ++c;
            }
        cnt[k + 1] = c;
    }
    scan();
    grow(next);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < n; ++k) {
        if (!todiv[k]) continue;
        int id = cnt[k + 1];
        for (int q = aptr[k]; q < aptr[k + 1]; ++q) {
            int i2 = adj[q];
            if (!(i2 < k) || todiv[i2]) continue;
            int j = edge_of(i2, k);
            if (j < 0) continue;
            midpoint(i2, j, addx[id - base], addy[id - base]);
            adjnode[q] = id;
            int qi = slot_of(i2, k);
            if (qi >= 0) adjnode[qi] = id;
            ++id;
        }
    }
    // create_centernodes (mesh_utils.f90:203-230)
    std::vector<int> center(n, -1);
    for (int i = 0; i < n; ++i) cnt[i + 1] = todiv[i] ? 1 : 0;
    scan();
    grow(next);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        if (!todiv[i]) continue;
        const int *v = &eind[eptr[i]];
        double px = nx[v[0]] + nx[v[1]] + nx[v[2]] + nx[v[3]];
        double py = ny[v[0]] + ny[v[1]] + ny[v[2]] + ny[v[3]];
        center[i] = cnt[i + 1];
        addx[center[i] - base] = px / 4.0;
        addy[center[i] - base] = py / 4.0;
    }
    // create_singlenodes (mesh_utils.f90:232-267): edges without a neighbour
    std::vector<int> nbr_on_edge((size_t)n * 4, -1), single((size_t)n * 4, -1);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        int c = 0;
        if (todiv[i]) {
            for (int q = aptr[i]; q < aptr[i + 1]; ++q) {
                int j = edge_of(i, adj[q]);
                if (j >= 0 && j < 4) nbr_on_edge[(size_t)i * 4 + j] = q;   // last neighbour on the edge
            }
            for (int j = 0; j < 4; ++j) c += nbr_on_edge[(size_t)i * 4 + j] < 0;
        }
        cnt[i + 1] = c;
    }
    scan();
    grow(next);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        if (!todiv[i]) continue;
        int id = cnt[i + 1];
        for (int j = 0; j < 4; ++j) {
            if (nbr_on_edge[(size_t)i * 4 + j] >= 0) continue;
            midpoint(i, j, addx[id - base], addy[id - base]);
            single[(size_t)i * 4 + j] = id++;
        }
    }
    // select_newhanging (mesh_utils.f90:411-452)
    std::vector<uint8_t> ishang(n, 0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        if (todiv[i]) continue;
        for (int q = aptr[i]; q < aptr[i + 1]; ++q)
            if (todiv[adj[q]] && adjnode[q] >= 0) { ishang[i] = 1; break; }
    }
    // final_division (mesh_utils.f90:454-681): kept elements in order, then
    // per element in order its hanging version or its four children
    std::vector<int> kptr(n + 1, 0), aslot(n + 1, 0), acnt(n + 1, 0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        int kept = 0, ae = 0, an = 0;
        if (ishang[i]) {
            int toins[4] = {-1, -1, -1, -1};
            for (int q = aptr[i]; q < aptr[i + 1]; ++q)
                if (todiv[adj[q]] && adjnode[q] >= 0) {
                    int j = edge_of(i, adj[q]);
                    if (j >= 0 && j < 4) toins[j] = adjnode[q];
                }
            ae = 1;
            an = 4;
            for (int j = 0; j < 4; ++j) an += toins[j] >= 0;
        } else if (todiv[i]) {
            ae = 4;
            an = 16;
        } else {
            kept = eptr[i + 1] - eptr[i];
        }
        kptr[i + 1] = kept;
        aslot[i + 1] = ae;
        acnt[i + 1] = an;
    }
    for (int i = 0; i < n; ++i) { kptr[i + 1] += kptr[i]; aslot[i + 1] += aslot[i]; acnt[i + 1] += acnt[i]; }
    int nkept = 0;
    for (int i = 0; i < n; ++i) nkept += !(ishang[i] || todiv[i]);
    const int nel_new = nkept + aslot[n];
    const int off = kptr[n];   // slots of the kept elements
    std::vector<int> neptr(nel_new + 1, 0), neind((size_t)off + acnt[n]), nemat(nel_new);
    std::vector<uint8_t> nediv((size_t)off + acnt[n], 0);
    // kept element index = rank among kept elements
    std::vector<int> krank(n + 1, 0);
    for (int i = 0; i < n; ++i) krank[i + 1] = krank[i] + !(ishang[i] || todiv[i]);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        if (ishang[i] || todiv[i]) {
            int e0 = nkept + aslot[i];
            int o = off + acnt[i];
            if (ishang[i]) {
                int toins[4] = {-1, -1, -1, -1};
                for (int q = aptr[i]; q < aptr[i + 1]; ++q) {
                    int k = adj[q];
                    if (!todiv[k] || adjnode[q] < 0) continue;
                    int j = edge_of(i, k);
                    if (j >= 0 && j < 4) toins[j] = adjnode[q];
                }
                const int *v = &eind[eptr[i]];
                for (int j = 0; j < 4; ++j) {
                    neind[o] = v[j]; nediv[o++] = 0;
                    if (toins[j] >= 0) { neind[o] = toins[j]; nediv[o++] = 1; }
                }
                neptr[e0 + 1] = o;
                nemat[e0] = emat[i];
            } else {
                int t[4];
                for (int j = 0; j < 4; ++j) {
                    int q = nbr_on_edge[(size_t)i * 4 + j];
                    t[j] = q < 0 ? single[(size_t)i * 4 + j] : adjnode[q];
                }
                const int *v = &eind[eptr[i]];
                int n1 = v[0], n2 = v[1], n3 = v[2], n4 = v[3], c = center[i];
                // material at the parent's opposite corner (mesh_utils.f90:622-649)
                double diff = ny[n3] - ny[n1];
                double p[4][2] = {{nx[n1] + diff, ny[n1] + diff}, {nx[n2] - diff, ny[n2] + diff},
                                  {nx[n3] - diff, ny[n3] - diff}, {nx[n4] + diff, ny[n4] - diff}};
                int kids[4][4] = {{n1, t[0], c, t[3]}, {t[0], n2, t[1], c}, {c, t[1], n3, t[2]}, {t[3], c, t[2], n4}};
                for (int q = 0; q < 4; ++q) {
                    for (int j = 0; j < 4; ++j) { neind[o] = kids[q][j]; nediv[o++] = 0; }
                    neptr[e0 + q + 1] = o;
                    nemat[e0 + q] = material_prop(p[q][0], p[q][1]);
                }
            }
        } else {
            const int e0 = krank[i];
            int o = kptr[i];
            for (int j = eptr[i]; j < eptr[i + 1]; ++j) { neind[o] = eind[j]; nediv[o++] = ediv[j]; }
            neptr[e0 + 1] = o;
            nemat[e0] = emat[i];
        }
    }
    eptr.swap(neptr); eind.swap(neind); ediv.swap(nediv); emat.swap(nemat);
    nx.insert(nx.end(), addx.begin(), addx.end());
    ny.insert(ny.end(), addy.begin(), addy.end());
    return true;
}

// setup_hanging (model.f90:654-675): (hanging, previous, next) per ediv slot.
void Model::setup_hanging() {
    hanging.clear();
    for (int i = 0; i < ne(); ++i)
        for (int j = eptr[i]; j < eptr[i + 1]; ++j)
            if (ediv[j]) {
                hanging.push_back(eind[j] + 1);
                hanging.push_back(eind[j - 1] + 1);
                hanging.push_back((j + 1 < eptr[i + 1] ? eind[j + 1] : eind[eptr[i]]) + 1);
            }
}

// create_absorbingbc (model.f90:1080-1096): XDIR on the sides wins at corners.
void Model::create_absorbingbc() {
    double left = 0.0 * blength, right = (double)(totcols - 1) * blength, top = (double)(totrows - 1) * blength;
    absorbing.assign(nx.size(), 0);
    for (size_t i = 0; i < nx.size(); ++i) {
        if (realequal(nx[i], left) || realequal(nx[i], right)) absorbing[i] = 2;
        else if (realequal(ny[i], top)) absorbing[i] = 1;
    }
}

// wave_elems (model.f90:1015-1045)
void Model::wave_elems() {
    seismic.clear();
    if (!is_wave) return;
    for (int e = 0; e < ne(); ++e) {
        int c[4];
        corners(e, c);
        int kind = 0;
        if (realequal(nx[c[1]], wleft) && realequal(ny[c[1]], wtop)) kind = 6;             // SE_CORNL
        else if (realequal(nx[c[0]], wright) && realequal(ny[c[0]], wtop)) kind = 5;       // SE_CORNR
        else if (realequal(nx[c[1]], wleft) && realunder(ny[c[1]], wtop)) kind = 2;        // SE_SVERL
        else if (realequal(nx[c[0]], wright) && realunder(ny[c[0]], wtop)) kind = 4;       // SE_SVERR
        else if (realover(nx[c[1]], wleft) && realunder(nx[c[0]], wright) && realequal(ny[c[0]], wtop)) kind = 1;  // SE_SHORI
        if (kind) { seismic.push_back(e + 1); seismic.push_back(kind); }
    }
}

// HETEROGENEITY: extension: every element inside the DRM box gets its own
// material with vp, vs scaled by exp(sigma*z1) and rho by exp(sigma*z2)
// (z ~ N(0,1), std::mt19937_64 seeded, factors clamped to [0.7, 1.3]).
void Model::apply_heterogeneity() {
    if (!(deck.het_sigma > 0)) return;
    std::mt19937_64 rng(deck.het_seed);
    std::normal_distribution<double> nd(0.0, 1.0);
    for (int e = 0; e < ne(); ++e) {
        double z1 = nd(rng), z2 = nd(rng);
        int c[4];
        corners(e, c);
        double cx = (nx[c[0]] + nx[c[1]] + nx[c[2]] + nx[c[3]]) / 4.0;
        double cy = (ny[c[0]] + ny[c[1]] + ny[c[2]] + ny[c[3]]) / 4.0;
        if (inside_soil(cx, cy)) continue;
        double fv = std::min(1.3, std::max(0.7, std::exp(deck.het_sigma * z1)));
        double fr = std::min(1.3, std::max(0.7, std::exp(deck.het_sigma * z2)));
        const double *m0 = &matconst[5 * (emat[e] - 1)];
        double vp = m0[3] * fv, vs = m0[4] * fv, rho = m0[2] * fr, mu, lam;
        v_to_lame(vp, vs, rho, &mu, &lam);
        matconst.push_back(mu); matconst.push_back(lam); matconst.push_back(rho);
        matconst.push_back(vp); matconst.push_back(vs);
        emat[e] = (int)(matconst.size() / 5);
    }
}

// recalculate_deltat (communicator.f90:1629-1662) + io_interval.
void Model::recalculate_deltat() {
    double mindt = deltat;
    double hmin = std::numeric_limits<double>::infinity(), hmax = 0;
    for (int e = 0; e < ne(); ++e) {
        double h = elength(e);
        hmin = std::min(hmin, h); hmax = std::max(hmax, h);
        double eldt = (h / matconst[5 * (emat[e] - 1) + 3]) / deck.sperlen;  // recalcstep
        mindt = std::min(mindt, eldt);
    }
    deltat = mindt;
    nsteps = (int)(duration / deltat);
    nsteps_deck = nsteps;
    io_interval = (int)(deck.inttime / deltat);
    inttime = deltat * io_interval;
    min_h = hmin; max_h = hmax;
    nlevels = 1 + (int)std::lround(std::log2(hmax / hmin));
}

// find_highest (visualization.f90:286-305) with highest_quadtree
// (quadtree.f90:253-291): the element reached first when the tree is walked
// towards the surface, i.e. the smallest top depth among elements whose x span
// holds x (tolerant compares); equal tops resolve to the right-hand element.
int Model::find_receivers() {
    recv_xy.clear(); recv_elem.clear();
    if (!deck.have_recv) return 0;
    if (!(deck.rdist > 0)) return fail(EXFEM_E_ARG, "RECEIVERS: dist must be positive");
    int np = (int)((deck.rxmax - deck.rxmin) / deck.rdist) + 1;
    if (np <= 0 || np > 1000000) return fail(EXFEM_E_ARG, "RECEIVERS: bad receiver count");
    // bucket elements by base-grid column for a fast search
    int ncol = totcols;
    std::vector<std::vector<int>> col(ncol + 1);
    for (int e = 0; e < ne(); ++e) {
        int c[4];
        corners(e, c);
        int a = (int)std::floor(nx[c[0]] / blength - 1e-6), b = (int)std::floor(nx[c[2]] / blength + 1e-6);
        for (int k = std::max(a, 0); k <= std::min(b, ncol); ++k) col[k].push_back(e);
    }
    for (int i = 1; i <= np; ++i) {
        double x = deck.rxmin + (deck.rdist * (double)i);
        int k = std::min(std::max((int)std::floor(x / blength), 0), ncol);
        int best = -1;
        double by = 0, bx = 0;
        for (int kk = std::max(k - 1, 0); kk <= std::min(k + 1, ncol); ++kk)
            for (int e : col[kk]) {
                int c[4];
                corners(e, c);
                if (realover(x, nx[c[2]]) || realunder(x, nx[c[0]])) continue;
                double top = ny[c[0]];
                if (best < 0 || realunder(top, by) || (realequal(top, by) && nx[c[0]] > bx) ||
                    (realequal(top, by) && nx[c[0]] == bx && e < best)) {
                    best = e; by = top; bx = nx[c[0]];
                }
            }
        if (best < 0) return fail(EXFEM_E_ARG, "RECEIVERS: receiver " + std::to_string(i) + " is outside the mesh");
        recv_xy.push_back(x);
        recv_xy.push_back(by);
        recv_elem.push_back(best + 1);
    }
    return 0;
}

void Model::export_arrays() {
    x_eptr.resize(eptr.size());
    for (size_t i = 0; i < eptr.size(); ++i) x_eptr[i] = eptr[i] + 1;
    x_eind.resize(eind.size());
    for (size_t i = 0; i < eind.size(); ++i) x_eind[i] = eind[i] + 1;
    x_nodes.resize(2 * nx.size());
    for (size_t i = 0; i < nx.size(); ++i) { x_nodes[2 * i] = nx[i]; x_nodes[2 * i + 1] = ny[i]; }
}

int build(const char *text, Model &m) {
    int rc = parse_deck(text, m.deck);
    if (rc) return rc;
    m.nmat_base = m.deck.nmats;
    if ((rc = setup_materials(m.deck, m.matconst))) return rc;
    if ((rc = m.setup_problem_params())) return rc;
    m.is_wave = m.deck.prob.compare(0, 4, "WAVE") == 0;
    if (m.is_wave) {
        if (m.deck.pparams.size() < 9) return fail(EXFEM_E_ARG, "PROBLEM: WAVE needs 9 parameters");
        int mat = (int)m.deck.pparams[4];
        if (mat < 1 || mat > m.nmat_base) return fail(EXFEM_E_ARG, "PROBLEM: exterior material out of range");
        if (m.deck.prob != "WAVEP " && m.deck.prob != "WAVESV")
            return fail(EXFEM_E_UNSUPPORTED, "PROBLEM: only WAVEP and WAVESV are on the accelerated path");
        m.init_wave();
        if (m.wcols < 1 || m.wrows < 1 || !(m.wright > m.wleft))
            return fail(EXFEM_E_ARG, "PROBLEM: DRM box does not fit the domain");
        if (m.deck.have_rhs) m.waves = m.deck.rhs;
        else {
            exfem_wave w{};
            w.kind = (m.deck.prob == "WAVEP ") ? EXFEM_WAVE_P : EXFEM_WAVE_SV;
            w.t0 = m.deck.pparams[5]; w.angle = m.deck.pparams[6];
            w.amp = m.deck.pparams[7]; w.freq = m.deck.pparams[8];
            m.waves.push_back(w);
        }
    } else if (m.deck.prob == "POINTN" || m.deck.prob == "POINTD") {
        // setup_point_source (model.f90:1051-1078): pparams = (amplitude,
        // sigma, start time, distance, x1, y1, x2, y2, ...)
        const std::vector<double> &pp = m.deck.pparams;
        if (pp.size() < 6) return fail(EXFEM_E_ARG, "PROBLEM: POINTN/POINTD need amplitude, sigma, start, distance and a point");
        if (!(pp[1] > 0)) return fail(EXFEM_E_ARG, "PROBLEM: point source sigma must be positive");
        m.point_kind = (m.deck.prob == "POINTN") ? EXFEM_POINT_FORCE : EXFEM_POINT_DISP;
        m.point_amp = pp[0];
        m.point_sigma = pp[1];
        m.point_t0 = pp[2];
        m.point_dist = pp[3];
        if (m.deck.have_rhs) return fail(EXFEM_E_ARG, "RHS: right-hand sides are plane waves; a point-source problem has one");
    } else {
        return fail(EXFEM_E_UNSUPPORTED, "PROBLEM: only WAVEP, WAVESV, POINTN and POINTD are on the accelerated path");
    }
    m.initial_mesh();
    // explicit.f90:42-52: cut, (redistribute: no-op on one rank), divide
    for (int pass = 0; pass < 32; ++pass) {
        m.cut_geom();
        if (!m.divide_pass()) break;
        if (m.ne() > 60000000) return fail(EXFEM_E_ARG, "mesh exceeds 6e7 elements");
    }
    for (int e = 0; e < m.ne(); ++e) {
        int c[4];
        if (!m.corners(e, c)) return fail(EXFEM_E_MESH, "element without four non-hanging corners");
    }
    m.setup_hanging();
    m.create_absorbingbc();
    m.wave_elems();
    m.setup_point_source();
    m.apply_heterogeneity();
    m.recalculate_deltat();
    if (m.io_interval < 1) return fail(EXFEM_E_ARG, "TIME: save interval shorter than the time step");
    if ((rc = m.find_receivers())) return rc;
    m.export_arrays();
    return 0;
}

template <typename T>
bool fwrite_all(FILE *f, const T *p, size_t n) { return std::fwrite(p, sizeof(T), n, f) == n; }

// ---------------------------------------------------- element quadtree ----
// Restatement of order_quadtree/search_quadtree (quadtree.f90:21-251):
// nodes split their elements about a centre snapped to the base length (or
// to the halved length that still fits the box), left/right by the lower
// x corner and down/up by the lower y corner; a leaf holds one element.
inline double realfloor(double a) { return std::floor(a + U_TOL); }      // utilities.f90:177-181
inline double realceiling(double a) { return std::ceil(a - U_TOL); }     // utilities.f90:183-187

struct QTree {
    struct Node {
        double cx = 0, cy = 0;
        int elem = -1;                 // 0-based leaf element, -1 inner node
        int child[4] = {-1, -1, -1, -1};   // downleft, upleft, downright, upright
    };
    std::vector<Node> nodes;
    const Model *m = nullptr;

    void box(int e, double &x0, double &y0, double &x1, double &y1) const {
        int c[4];
        m->corners(e, c);
        x0 = m->nx[c[0]]; y0 = m->ny[c[0]]; x1 = m->nx[c[2]]; y1 = m->ny[c[2]];
    }
    // pivot split of elems[lo, hi) by the lower corner against centre v (axis 0 = x)
    int split(std::vector<int> &el, int lo, int hi, int axis, double v) const {
        int st = lo, en = hi - 1;
        while (st <= en) {
            double a0, b0, a1, b1, c0, d0, c1, d1;
            box(el[st], a0, b0, a1, b1);
            box(el[en], c0, d0, c1, d1);
            if (realover(v, axis == 0 ? a0 : b0)) { ++st; continue; }
            if (realunder(v, axis == 0 ? c1 : d1)) { --en; continue; }
            std::swap(el[st], el[en]);
            ++st;
            --en;
        }
        return st;
    }
    int build(std::vector<int> &el, int lo, int hi, int depth) {
        const int id = (int)nodes.size();
        nodes.emplace_back();
        if (hi - lo == 1 || depth > 200) { nodes[id].elem = el[lo]; return id; }
        const double inf = std::numeric_limits<double>::infinity();
        double mn[2] = {inf, inf}, mx[2] = {-inf, -inf};
        for (int i = lo; i < hi; ++i) {
            double x0, y0, x1, y1;
            box(el[i], x0, y0, x1, y1);
            mn[0] = std::min(mn[0], x0); mn[1] = std::min(mn[1], y0);
            mx[0] = std::max(mx[0], x1); mx[1] = std::max(mx[1], y1);
        }
        double dist[2] = {mx[0] - mn[0], mx[1] - mn[1]};
        const double bl = m->blength;
        double len = bl;
        if (!(realunder(bl, dist[0]) || realunder(bl, dist[1]))) {
            len = bl / 2.0;
            while (!realunder(len, dist[0]) && !realunder(len, dist[1])) len = len / 2.0;
        }
        for (int a = 0; a < 2; ++a) {
            mn[a] = realfloor(mn[a] / len) * len;
            mx[a] = realceiling(mx[a] / len) * len;
            dist[a] = realfloor(((mx[a] - mn[a]) / 2.0) / len) * len;
        }
        const double cx = mn[0] + dist[0], cy = mn[1] + dist[1];
        nodes[id].cx = cx;
        nodes[id].cy = cy;
        const int mid = split(el, lo, hi, 0, cx);
        if (mid > lo) {
            const int s = split(el, lo, mid, 1, cy);
            if (s > lo) { int k = build(el, lo, s, depth + 1); nodes[id].child[0] = k; }
            if (s < mid) { int k = build(el, s, mid, depth + 1); nodes[id].child[1] = k; }
        }
        if (mid < hi) {
            const int s = split(el, mid, hi, 1, cy);
            if (s > mid) { int k = build(el, mid, s, depth + 1); nodes[id].child[2] = k; }
            if (s < hi) { int k = build(el, s, hi, depth + 1); nodes[id].child[3] = k; }
        }
        return id;
    }
    void build(const Model &model) {
        m = &model;
        nodes.clear();
        std::vector<int> el(model.ne());
        for (int e = 0; e < model.ne(); ++e) el[e] = e;
        if (!el.empty()) build(el, 0, (int)el.size(), 0);
    }
    // inside_element (model.f90:176-186)
    bool inside(int e, double px, double py) const {
        double x0, y0, x1, y1;
        box(e, x0, y0, x1, y1);
        return !realunder(px, x0) && !realunder(py, y0) && !realover(px, x1) && !realover(py, y1);
    }
    // search_quadtree: 0-based element or -1
    int search(double px, double py) const {
        int t = nodes.empty() ? -1 : 0;
        while (t >= 0) {
            const Node &n = nodes[t];
            if (n.elem >= 0) return inside(n.elem, px, py) ? n.elem : -1;
            const bool ux = px < n.cx, uy = py < n.cy;
            t = ux ? (uy ? n.child[0] : n.child[1]) : (uy ? n.child[2] : n.child[3]);
        }
        return -1;
    }
};

// base64 of write_vtk_unst_field (io.cpp:623-663)
const char B64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";

std::string b64(const unsigned char *in, size_t n) {
    std::string out;
    out.reserve(4 * ((n + 2) / 3));
    for (size_t i = 0; i < n;) {
        unsigned a = i < n ? in[i++] : 0, b = i < n ? in[i++] : 0, c = i < n ? in[i++] : 0;
        unsigned t = (a << 16) + (b << 8) + c;
        out += B64[(t >> 18) & 63]; out += B64[(t >> 12) & 63]; out += B64[(t >> 6) & 63]; out += B64[t & 63];
    }
    static const int pad[3] = {0, 2, 1};
    for (int i = 0; i < pad[n % 3]; ++i) out[out.size() - 1 - i] = '=';
    return out;
}

// num_to_base64: the four little-endian bytes of an int as 8 characters
std::string b64_len(int v) {
    unsigned char ch[4];
    std::memcpy(ch, &v, 4);
    unsigned t = ((unsigned)ch[0] << 16) + ((unsigned)ch[1] << 8) + ch[2];
    std::string out;
    out += B64[(t >> 18) & 63]; out += B64[(t >> 12) & 63]; out += B64[(t >> 6) & 63]; out += B64[t & 63];
    t = (unsigned)ch[3] << 16;
    out += B64[(t >> 18) & 63]; out += B64[(t >> 12) & 63];
    out += "==";
    return out;
}

// pointdata_to_base64: (x, y) pairs as float (x, y, 0) triples
std::string b64_points(int n, const double *p) {
    std::vector<float> f((size_t)3 * n);
    for (int i = 0; i < n; ++i) { f[3 * (size_t)i] = (float)p[2 * (size_t)i]; f[3 * (size_t)i + 1] = (float)p[2 * (size_t)i + 1]; f[3 * (size_t)i + 2] = 0.0f; }
    return b64(reinterpret_cast<const unsigned char *>(f.data()), f.size() * sizeof(float));
}

struct Grid : exfem_grid {
    std::vector<double> pts, mat;
    std::vector<int> el, ptr, ind;
};

}  // namespace

struct exfem_model : Model {};

extern "C" {

int exfem_model_build(const char *deck_text, exfem_model **out) {
    if (!out) return fail(EXFEM_E_ARG, "out is NULL");
    *out = nullptr;
    exfem_model *m = nullptr;
    try {
        m = new exfem_model();
        int rc = build(deck_text, *m);
        if (rc) { delete m; return rc; }
    } catch (const std::bad_alloc &) {
        delete m;
        return fail(EXFEM_E_NOMEM, "host allocation failed while building the model");
    } catch (const std::exception &ex) {
        delete m;
        return fail(EXFEM_E_ARG, ex.what());
    }
    *out = m;
    return 0;
}

const char *exfem_model_error(void) { return g_err.c_str(); }

void exfem_model_views(const exfem_model *m, exfem_mesh *mesh, exfem_problem *prob) {
    if (mesh) {
        mesh->nelems = m->ne();
        mesh->nnodes = (int)m->nx.size();
        mesh->eptr = m->x_eptr.data();
        mesh->eind = m->x_eind.data();
        mesh->ediv = m->ediv.data();
        mesh->nodes = m->x_nodes.data();
        mesh->ematprop = m->emat.data();
    }
    if (prob) {
        std::memset(prob, 0, sizeof(*prob));
        prob->nmat = (int)(m->matconst.size() / 5);
        prob->matconst = m->matconst.data();
        prob->absorbing = m->absorbing.data();
        prob->nhanging = (int)(m->hanging.size() / 3);
        prob->hanging = m->hanging.data();
        prob->nseismic = (int)(m->seismic.size() / 2);
        prob->seismic = m->seismic.data();
        prob->deltat = m->deltat;
        prob->nsteps = m->nsteps;
        prob->io_interval = m->io_interval;
        prob->worigin[0] = m->worigin[0];
        prob->worigin[1] = m->worigin[1];
        prob->wbox[0] = m->wleft;
        prob->wbox[1] = m->wright;
        prob->wbox[2] = m->wtop;
        prob->walpha = m->walpha;
        prob->wbeta = m->wbeta;
        prob->nrhs = std::max(1, (int)m->waves.size());
        prob->waves = m->waves.empty() ? nullptr : m->waves.data();
        prob->point_kind = m->point_kind;
        prob->npoint = (int)m->point_nodes.size();
        prob->point_nodes = m->point_nodes.empty() ? nullptr : m->point_nodes.data();
        prob->point_amp = m->point_amp;
        prob->point_sigma = m->point_sigma;
        prob->point_t0 = m->point_t0;
        prob->nrecv = (int)m->recv_elem.size();
        prob->recv_xy = m->recv_xy.data();
        prob->recv_elem = m->recv_elem.data();
    }
}

void exfem_model_get_info(const exfem_model *m, exfem_model_info *info) {
    std::memset(info, 0, sizeof(*info));
    info->width = m->deck.width; info->height = m->deck.height;
    info->duration = m->duration; info->inttime = m->inttime; info->chper = m->deck.chper;
    info->nperlen = m->deck.nperlen; info->sperlen = m->deck.sperlen;
    info->blength = m->blength; info->mlength = m->mlength;
    info->totcols = m->totcols; info->totrows = m->totrows;
    info->wrows = m->wrows; info->wcols = m->wcols;
    info->nmat_base = m->nmat_base; info->nmat = (int)(m->matconst.size() / 5);
    info->nelems = m->ne(); info->nnodes = (int)m->nx.size();
    info->nhanging = (int)(m->hanging.size() / 3); info->nseismic = (int)(m->seismic.size() / 2);
    info->nrecv = (int)m->recv_elem.size(); info->nrhs = std::max(1, (int)m->waves.size());
    info->nsteps = m->nsteps; info->io_interval = m->io_interval; info->deltat = m->deltat;
    info->nlevels = m->nlevels; info->min_h = m->min_h; info->max_h = m->max_h;
}

int exfem_model_set_nsteps(exfem_model *m, int nsteps) {
    if (!m || nsteps < 0) return fail(EXFEM_E_ARG, "bad nsteps");
    if (nsteps > m->nsteps_deck)
        return fail(EXFEM_E_ARG, "deck gives " + std::to_string(m->nsteps_deck) + " steps, " +
                                     std::to_string(nsteps) + " requested");
    m->nsteps = nsteps;
    return 0;
}

int exfem_model_save_mesh(const exfem_model *m, const char *path) {
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(EXFEM_E_ARG, std::string("cannot open ") + path);
    int ne = m->ne(), nn = (int)m->nx.size();
    // save_binmesh writes eptr[nelems] entries of eind and ediv (io.cpp:354,
    // 357); with 1-based offsets that is one more than the connectivity holds,
    // so the file carries one trailing pad entry in each array.
    const int pad_i = 0;
    const unsigned char pad_b = 0;
    bool ok = fwrite_all(f, &ne, 1) && fwrite_all(f, m->x_eptr.data(), m->x_eptr.size()) &&
              fwrite_all(f, m->x_eind.data(), m->x_eind.size()) && fwrite_all(f, &pad_i, 1);
    // ediv is Fortran logical*1 / C bool: one byte per slot
    ok = ok && fwrite_all(f, m->ediv.data(), m->ediv.size()) && fwrite_all(f, &pad_b, 1);
    ok = ok && fwrite_all(f, &nn, 1) && fwrite_all(f, m->x_nodes.data(), m->x_nodes.size());
    std::fclose(f);
    return ok ? 0 : fail(EXFEM_E_ARG, "short write");
}

int exfem_write_mass(const char *path, int ndofs, const double *mass) {
    FILE *f = std::fopen(path, "wb");
    if (!f) return fail(EXFEM_E_ARG, std::string("cannot open ") + path);
    bool ok = fwrite_all(f, &ndofs, 1) && fwrite_all(f, mass, (size_t)ndofs);
    std::fclose(f);
    return ok ? 0 : fail(EXFEM_E_ARG, "short write");
}

int exfem_write_step(const char *path, int append, int step, int ndofs, const double *u) {
    FILE *f = std::fopen(path, append ? "ab" : "wb");
    if (!f) return fail(EXFEM_E_ARG, std::string("cannot open ") + path);
    bool ok = fwrite_all(f, &step, 1) && fwrite_all(f, &ndofs, 1) && fwrite_all(f, u, (size_t)ndofs);
    std::fclose(f);
    return ok ? 0 : fail(EXFEM_E_ARG, "short write");
}

int exfem_write_sheet(const char *path, int npoints, const double *points, int nsave, const double *field,
                      double samp) {
    FILE *f = std::fopen(path, "w");
    if (!f) return fail(EXFEM_E_ARG, std::string("cannot open ") + path);
    std::fprintf(f, "POINTS = [ ");
    // save_sheet_points passes 2*npoints values: (x, depth) per receiver (io_utils.f90:479-486)
    for (int i = 0; i < 2 * npoints; ++i) std::fprintf(f, "%.10lf ", points[i]);
    std::fprintf(f, " ];");
    std::fprintf(f, "\nFIELD = [ ");
    for (int s = 0; s < nsave; ++s) {
        for (int i = 0; i < 2 * npoints; ++i) std::fprintf(f, "%lf ", field[(size_t)s * 2 * npoints + i]);
        std::fprintf(f, "\n");
    }
    std::fprintf(f, " ];\n");
    std::fprintf(f, "SAMP = %lf ;", samp);
    std::fclose(f);
    return 0;
}

int exfem_model_grid(const exfem_model *m, double xmin, double xmax, double ymin, double ymax, double dist,
                     exfem_grid **out) {
    if (!m || !out || !(dist > 0) || !(xmax >= xmin) || !(ymax >= ymin)) return fail(EXFEM_E_ARG, "bad grid");
    *out = nullptr;
    // visu_points (visualization.f90:129-154)
    const int nx = (int)((xmax - xmin) / dist), ny = (int)((ymax - ymin) / dist);
    if ((double)(nx + 1) * (ny + 1) > 2.0e8) return fail(EXFEM_E_ARG, "grid over 2e8 points");
    Grid *g = new (std::nothrow) Grid();
    if (!g) return fail(EXFEM_E_NOMEM, "grid");
    const int np = (nx + 1) * (ny + 1);
    g->pts.resize(2 * (size_t)np);
    int k = 0;
    for (int i = 0; i <= nx; ++i)
        for (int j = 0; j <= ny; ++j, ++k) {
            g->pts[2 * (size_t)k] = xmin + (double)i * dist;
            g->pts[2 * (size_t)k + 1] = ymin + (double)j * dist;
        }
    QTree qt;
    qt.build(*m);
    g->el.assign(np, 0);
    g->mat.assign(2 * (size_t)np, 0.0);
    int found = 0;
    for (int p = 0; p < np; ++p) {
        const double px = g->pts[2 * (size_t)p], py = g->pts[2 * (size_t)p + 1];
        const int e = qt.search(px, py);
        if (e < 0) continue;
        g->el[p] = e + 1;
        ++found;
        const int prop = m->material_prop(px, py);   // visu_material
        g->mat[2 * (size_t)p] = (double)prop;
        g->mat[2 * (size_t)p + 1] = m->matconst[5 * (size_t)(prop - 1) + 3];
    }
    // create_struct_mesh (mesh_utils.f90:846-878)
    g->ptr.assign((size_t)nx * ny + 1, 1);
    g->ind.resize(4 * (size_t)nx * ny);
    int c = 0;
    for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j, ++c) {
            g->ptr[c + 1] = g->ptr[c] + 4;
            int *q = &g->ind[4 * (size_t)c];
            q[0] = (i - 1) * (ny + 1) + j;
            q[1] = i * (ny + 1) + j;
            q[2] = i * (ny + 1) + (j + 1);
            q[3] = (i - 1) * (ny + 1) + (j + 1);
        }
    g->nx = nx; g->ny = ny;
    g->origin[0] = xmin; g->origin[1] = ymin;
    g->space = dist;
    g->npoints = np;
    g->points = g->pts.data();
    g->elem = g->el.data();
    g->material = g->mat.data();
    g->ncells = nx * ny;
    g->eptr = g->ptr.data();
    g->eind = g->ind.data();
    g->nfound = found;
    *out = g;
    return 0;
}

void exfem_grid_free(exfem_grid *g) { delete static_cast<Grid *>(g); }

int exfem_write_vtu(const char *path, int ncells, const int *eptr, const int *eind, int npoints,
                    const double *points, const char *fieldname, const double *field) {
    if (!path || ncells < 0 || npoints < 0 || (ncells && (!eptr || !eind)) || (npoints && (!points || !field)) ||
        !fieldname)
        return fail(EXFEM_E_ARG, "bad vtu arguments");
    FILE *f = std::fopen(path, "w");
    if (!f) return fail(EXFEM_E_ARG, std::string("cannot open ") + path);
    const int nconn = ncells ? eptr[ncells] - 1 : 0;
    int off[6];
    off[0] = 0;
    off[1] = off[0] + 4 * (int)((((size_t)npoints * sizeof(float) * 3) + 2) / 3) + 8;
    off[2] = off[1] + 4 * (int)((((size_t)npoints * sizeof(float) * 3) + 2) / 3) + 8;
    off[3] = off[2] + 4 * (int)((((size_t)nconn * sizeof(int)) + 2) / 3) + 8;
    off[4] = off[3] + 4 * (int)((((size_t)ncells * sizeof(int)) + 2) / 3) + 8;
    off[5] = off[4] + 4 * (int)((((size_t)ncells * sizeof(int)) + 2) / 3) + 8;
    std::fprintf(f, "<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\">\n");
    std::fprintf(f, "<UnstructuredGrid>\n");
    std::fprintf(f, "<Piece NumberOfPoints=\"%d\" NumberOfCells=\"%d\">\n", npoints, ncells);
    std::fprintf(f, "<PointData>\n");
    std::fprintf(f, "<DataArray type=\"Float32\" Name=\"%s\"", fieldname);
    std::fprintf(f, " NumberOfComponents=\"3\" format=\"appended\" offset=\"%d\">\n", off[0]);
    std::fprintf(f, "\n</DataArray>\n");
    std::fprintf(f, "</PointData>\n");
    std::fprintf(f, "<CellData>\n");
    std::fprintf(f, "</CellData>\n");
    std::fprintf(f, "<Points>\n");
    std::fprintf(f, "<DataArray type=\"Float32\" Name=\"points\"");
    std::fprintf(f, " NumberOfComponents=\"3\" format=\"appended\" offset=\"%d\">\n", off[1]);
    std::fprintf(f, "\n</DataArray>\n");
    std::fprintf(f, "</Points>\n");
    std::fprintf(f, "<Cells>\n");
    std::fprintf(f, "<DataArray type=\"Int32\" Name=\"connectivity\" format=\"appended\" offset=\"%d\">\n", off[2]);
    std::fprintf(f, "\n</DataArray>\n");
    std::fprintf(f, "<DataArray type=\"Int32\" Name=\"offsets\" Format=\"appended\" offset=\"%d\">\n", off[3]);
    std::fprintf(f, "\n</DataArray>\n");
    std::fprintf(f, "<DataArray type=\"Int32\" Name=\"types\" Format=\"appended\" offset=\"%d\">\n", off[4]);
    std::fprintf(f, "\n</DataArray>\n");
    std::fprintf(f, "</Cells>\n");
    std::fprintf(f, "</Piece>\n");
    std::fprintf(f, "</UnstructuredGrid>\n\n");
    std::fprintf(f, "<AppendedData encoding=\"base64\">\n\n");
    std::fputc('_', f);
    // each block: its base64 length as an 8-character word, then the data
    std::string t = b64_points(npoints, field);
    std::fputs(b64_len((int)t.size()).c_str(), f);
    std::fputs(t.c_str(), f);
    t = b64_points(npoints, points);
    std::fputs(b64_len((int)t.size()).c_str(), f);
    std::fputs(t.c_str(), f);
    // mesh_to_base64: 0-based connectivity, end offsets
    std::vector<int> conn(nconn), offs(ncells);
    for (int i = 0; i < ncells; ++i) {
        offs[i] = eptr[i + 1] - 1;
        for (int j = eptr[i] - 1; j < eptr[i + 1] - 1; ++j) conn[j] = eind[j] - 1;
    }
    t = b64(reinterpret_cast<const unsigned char *>(conn.data()), conn.size() * sizeof(int));
    std::fputs(b64_len((int)t.size()).c_str(), f);
    std::fputs(t.c_str(), f);
    t = b64(reinterpret_cast<const unsigned char *>(offs.data()), offs.size() * sizeof(int));
    const std::string offlen = b64_len((int)t.size());
    std::fputs(offlen.c_str(), f);
    std::fputs(t.c_str(), f);
    // types: the offsets' length word again, then VTK_POLYGON (7) in groups
    // of three cells plus the remainder, as io.cpp:827-833 writes them
    std::fputs(offlen.c_str(), f);
    for (int i = 0; i < ncells; i += 3) std::fputs("BwAAAAcAAAAHAAAA", f);
    if (ncells % 3 == 1) std::fputs("BwAAAA==", f);
    else if (ncells % 3 == 2) std::fputs("BwAAAAcAAAA=", f);
    std::fprintf(f, "\n\n</AppendedData>\n");
    std::fprintf(f, "</VTKFile>\n");
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    return ok ? 0 : fail(EXFEM_E_ARG, std::string("write failed: ") + path);
}

void exfem_model_free(exfem_model *m) { delete m; }

}  // extern "C"
