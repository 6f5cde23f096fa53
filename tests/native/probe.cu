// probe.cu — test-only host build of the library's plan builder and of its
// __host__ __device__ arithmetic, so the CPU suite can check both without a
// GPU.  Compiled by tests/native_probe.py with nvcc into tests/native/_build.
#include <omp.h>

#include <cstring>
#include <string>

#include "exfem_device.cuh"
#include "exfem_plan.h"
#include "exfem_tc.cuh"

using namespace exfem;

namespace {
std::string g_err;

DevWave to_dev(const WaveConst &w) {
    DevWave d;
    d.kind = w.kind; d.alpha = w.alpha; d.beta = w.beta; d.fp = w.fp;
    d.sine = w.sine; d.cose = w.cose; d.sinf = w.sinf; d.cosf = w.cosf;
    d.amp0 = w.amp0; d.wa1 = w.wa1; d.wb1 = w.wb1;
    for (int k = 0; k < 6; ++k) d.wui[k] = w.wui[k];
    d.t0 = w.t0;
    d.inv_alpha = 1.0 / w.alpha;
    d.inv_beta = 1.0 / w.beta;
    return d;
}
}  // namespace

extern "C" {

const char *probe_error(void) { return g_err.c_str(); }

// calck's 64 entries as formulas (formulation.f90:276-313) against the matrix
// the FP64 kernels rebuild from calck_values' six host values: the index of
// the first entry whose bits differ, or -1 when all 64 match.
int probe_calck_check(double m, double l) {
    const double f[64] = {
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
    double kv[6], k[64];
    calck_values(m, l, kv);
    calck(kv, k);
    for (int i = 0; i < 64; ++i)
        if (std::memcmp(&f[i], &k[i], sizeof(double)) != 0) return i;
    return -1;
}

// Threads the plan builder's parallel loops use from here on.
void probe_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }

// The state offset of (node n, dof d, rhs r) for R right-hand sides in
// groups of lg (row_off / state_at).
long long probe_state_at(int R, int lg, long long n, int d, int r) {
    DevModel m{};
    m.R = R;
    m.lg = lg;
    return (long long)state_at(m, (size_t)n, d, r);
}

void probe_q4_ku(double A, double B, double C, double D, const double *ux, const double *uy, double *fx, double *fy) {
    q4_ku<double>(A, B, C, D, ux, uy, fx, fy);
}

void probe_q4_ku_corner(double A, double B, double C, double D, const double *ux, const double *uy, int c,
                        double *fx, double *fy) {
    q4_ku_corner<double>(A, B, C, D, ux, uy, c, *fx, *fy);
}

// -w times the corner force, through q4_fold + q4_corner_acc (from zero).
void probe_q4_corner_acc(double A, double B, double C, double D, const double *ux, const double *uy, int c, double w,
                         double *ax, double *ay) {
    const Q4Fold<double> f = q4_fold<double>(A, B, C, D, c, w);
    *ax = 0.0;
    *ay = 0.0;
    q4_corner_acc<double>(f, ux, uy, *ax, *ay);
}

void probe_q4_ku_f32(float A, float B, float C, float D, const float *ux, const float *uy, float *fx, float *fy) {
    q4_ku<float>(A, B, C, D, ux, uy, fx, fy);
}

void probe_drm_forces(const double *k4, double mass, int kind, const double *u0, const double *a0, double *p) {
    drm_forces<double>(k4, mass, drm_mask(kind), u0, a0, p);
}

int probe_planewave(int kind, double amp, double alpha, double beta, double angle, double freq, double t, double x1,
                    double x3, double *u6) {
    exfem_wave w{kind, amp, angle, freq, 0.0};
    WaveConst wc;
    int rc = init_wave_const(w, alpha, beta, wc, g_err);
    if (rc) return rc;
    DevWave d = to_dev(wc);
    double ux[3], uz[3];
    planewave(d, t, x1, x3, ux, uz);
    for (int c = 0; c < 3; ++c) { u6[2 * c] = ux[c]; u6[2 * c + 1] = uz[c]; }
    return 0;
}

// The FP32 free field of the FP32 form: u2 = (ux, uz), a2 = (ax, az).
int probe_planewave32(int kind, double amp, double alpha, double beta, double angle, double freq, double t, double x1,
                      double x3, float *u2, float *a2) {
    exfem_wave w{kind, amp, angle, freq, 0.0};
    WaveConst wc;
    int rc = init_wave_const(w, alpha, beta, wc, g_err);
    if (rc) return rc;
    DevWave d = to_dev(wc);
    planewave32(d, t, x1, x3, u2, a2);
    return 0;
}

// The displacement-only path used by the receivers.
int probe_planewave_u(int kind, double amp, double alpha, double beta, double angle, double freq, double t, double x1,
                      double x3, double *u2) {
    exfem_wave w{kind, amp, angle, freq, 0.0};
    WaveConst wc;
    int rc = init_wave_const(w, alpha, beta, wc, g_err);
    if (rc) return rc;
    DevWave d = to_dev(wc);
    planewave_u(d, t, x1, x3, u2[0], u2[1]);
    return 0;
}

void *probe_plan(const exfem_mesh *mesh, const exfem_problem *prob, int reorder) {
    Plan *p = new Plan();
    int rc = build_plan(*mesh, *prob, reorder != 0, *p, g_err);
    if (rc) { delete p; return nullptr; }
    return p;
}

void probe_plan_free(void *h) { delete static_cast<Plan *>(h); }

// Sizes and copies of the plan arrays by name.
long long probe_plan_size(void *h, const char *name) {
    Plan &p = *static_cast<Plan *>(h);
    std::string n(name);
#define SZ(f) if (n == #f) return (long long)p.f.size();
    SZ(ref_of_node) SZ(node_of_ref) SZ(ref_of_elem) SZ(econn) SZ(ecoef) SZ(emass) SZ(edamp) SZ(edampv)
    SZ(tptr) SZ(tlist) SZ(dptr) SZ(dlist) SZ(mfull_ref) SZ(inv_mfull) SZ(nmass) SZ(ndamp) SZ(hang)
    SZ(s_elem) SZ(s_kind) SZ(rnode) SZ(rw) SZ(rsoil) SZ(rxy) SZ(lptr) SZ(llist) SZ(ownptr) SZ(ownlist)
    SZ(ecoef32) SZ(ecoef2) SZ(emulam) SZ(mfull_int) SZ(elem_of_ref) SZ(nxy) SZ(odptr) SZ(odlist)
#undef SZ
    if (n == "scalars") return 8;
    return -1;
}

int probe_plan_copy(void *h, const char *name, void *out) {
    Plan &p = *static_cast<Plan *>(h);
    std::string n(name);
#define CP(f) if (n == #f) { if (!p.f.empty()) std::memcpy(out, p.f.data(), p.f.size() * sizeof(p.f[0])); return 0; }
    CP(ref_of_node) CP(node_of_ref) CP(ref_of_elem) CP(econn) CP(ecoef) CP(emass) CP(edamp) CP(edampv)
    CP(tptr) CP(tlist) CP(dptr) CP(dlist) CP(mfull_ref) CP(inv_mfull) CP(nmass) CP(ndamp) CP(hang)
    CP(s_elem) CP(s_kind) CP(rnode) CP(rw) CP(rsoil) CP(rxy) CP(lptr) CP(llist) CP(ownptr) CP(ownlist)
    CP(ecoef32) CP(ecoef2) CP(emulam) CP(mfull_int) CP(elem_of_ref) CP(nxy) CP(odptr) CP(odlist)
#undef CP
    if (n == "scalars") {
        double *d = static_cast<double *>(out);
        d[0] = p.n_active; d[1] = p.n_hang; d[2] = p.a1; d[3] = p.a2; d[4] = p.a3; d[5] = p.dt; d[6] = p.nsave; d[7] = p.io;
        return 0;
    }
    return -1;
}

// Shared-memory tiles of a plan: fills sizes[0..3] = (ntiles, hmax, halo
// entries, tn) and, when the pointers are non-NULL, copies the arrays.
int probe_tiles(void *h, int tn, int *sizes, int *hptr, int *hlist, unsigned short *tslot, int *nslot, int *lslot) {
    Plan &p = *static_cast<Plan *>(h);
    Tiles T;
    int rc = build_tiles(p, tn, T, g_err);
    if (rc) return rc;
    sizes[0] = T.ntiles; sizes[1] = T.hmax; sizes[2] = (int)T.hlist.size(); sizes[3] = T.tn;
    if (hptr) std::memcpy(hptr, T.hptr.data(), T.hptr.size() * sizeof(int));
    if (hlist) std::memcpy(hlist, T.hlist.data(), T.hlist.size() * sizeof(int));
    if (tslot) std::memcpy(tslot, T.tslot.data(), T.tslot.size() * sizeof(unsigned short));
    if (nslot) std::memcpy(nslot, T.nslot.data(), T.nslot.size() * sizeof(int));
    if (lslot && !T.lslot.empty()) std::memcpy(lslot, T.lslot.data(), T.lslot.size() * sizeof(int));
    return 0;
}

// Element tiles of the tensor-core step (build_mma_tiles): sizes[0..2] =
// (ntiles, elements listed, most elements in a tile); nptr[ntiles + 1],
// eptr[ntiles + 1], elist and tj[terms] are copied when non-NULL.  Returns 0,
// or 1 when the builder refuses the model.
int probe_mma_tiles(void *h, int tn, int emax, int *sizes, int *nptr, int *eptr, int *elist, unsigned char *tj) {
    Plan &p = *static_cast<Plan *>(h);
    MmaTiles T;
    if (!build_mma_tiles(p, tn, emax, T, g_err)) return 1;
    sizes[0] = T.ntiles; sizes[1] = (int)T.elist.size(); sizes[2] = T.emax;
    if (nptr) std::memcpy(nptr, T.nptr.data(), T.nptr.size() * sizeof(int));
    if (eptr) std::memcpy(eptr, T.eptr.data(), T.eptr.size() * sizeof(int));
    if (elist && !T.elist.empty()) std::memcpy(elist, T.elist.data(), T.elist.size() * sizeof(int));
    if (tj && !T.tj.empty()) std::memcpy(tj, T.tj.data(), T.tj.size());
    return 0;
}

// The direct gather's slot records (build_node_slots): slot4[4 * n_active]
// and invm[n_active] when non-NULL; returns the marked node count, or -1
// when the builder refuses the model.
long long probe_node_slots(void *h, int *slot4, float *invm) {
    Plan &p = *static_cast<Plan *>(h);
    NodeSlots S;
    if (!build_node_slots(p, node_coef32(p), S, g_err)) return -1;
    if (slot4) std::memcpy(slot4, S.slot4.data(), S.slot4.size() * sizeof(int));
    if (invm) std::memcpy(invm, S.invm.data(), S.invm.size() * sizeof(float));
    return S.marked;
}

// The FP32 node coefficients (node_coef32): 4 per active node.
void probe_node_coef32(void *h, float *out) {
    Plan &p = *static_cast<Plan *>(h);
    const pvec<float> nc = node_coef32(p);
    std::memcpy(out, nc.data(), nc.size() * sizeof(float));
}

// The tensor-core step's B operand (tc_b_operand_q4): 256 floats, the tf32 hi
// tile then the lo tile, in the K-major core-matrix layout.
void probe_mma_btile(float *out) {
    const std::vector<float> b = tc_b_operand_q4();
    std::memcpy(out, b.data(), b.size() * sizeof(float));
}

// Halo runs of the tiles (the bulk copies of the pipelined step): fills
// rptr[ntiles + 1] and runs[2 * nruns] when non-NULL; returns nruns.
int probe_tile_runs(void *h, int tn, int *rptr, int *runs) {
    Plan &p = *static_cast<Plan *>(h);
    Tiles T;
    int rc = build_tiles(p, tn, T, g_err);
    if (rc) return rc;
    if (rptr) std::memcpy(rptr, T.rptr.data(), T.rptr.size() * sizeof(int));
    if (runs) std::memcpy(runs, T.runs.data(), T.runs.size() * sizeof(int));
    return (int)(T.runs.size() / 2);
}

// The bulk-copy pipeline's records (build_pipe_pack): sizes[0..4] = (hdr,
// runs, nrec, tpack words, tmax); the arrays are copied when non-NULL.
// Returns 0, or 1 when the model does not fit the formats.
int probe_pipe_pack(void *h, int tn, int max_runs, int *sizes, int *hdr, int *runs, int *nrec, int *tpack) {
    Plan &p = *static_cast<Plan *>(h);
    Tiles T;
    int rc = build_tiles(p, tn, T, g_err);
    if (rc) return rc;
    PipePack pk;
    if (!build_pipe_pack(p, T, max_runs, pk, g_err)) return 1;
    sizes[0] = (int)pk.hdr.size(); sizes[1] = (int)pk.runs.size(); sizes[2] = (int)pk.nrec.size();
    sizes[3] = (int)pk.tpack.size(); sizes[4] = pk.tmax;
    if (hdr) std::memcpy(hdr, pk.hdr.data(), pk.hdr.size() * sizeof(int));
    if (runs) std::memcpy(runs, pk.runs.data(), pk.runs.size() * sizeof(int));
    if (nrec) std::memcpy(nrec, pk.nrec.data(), pk.nrec.size() * sizeof(int));
    if (tpack) std::memcpy(tpack, pk.tpack.data(), pk.tpack.size() * sizeof(int));
    return 0;
}

// Free-field displacement+acceleration at a point for RHS r of a plan
// (what k_drm evaluates).
void probe_plan_wave(void *h, int r, double t, double x1, double x3, double *u6) {
    Plan &p = *static_cast<Plan *>(h);
    DevWave d = to_dev(p.waves[r]);
    double ux[3], uz[3];
    planewave(d, t - d.t0, x1, x3, ux, uz);
    for (int c = 0; c < 3; ++c) { u6[2 * c] = ux[c]; u6[2 * c + 1] = uz[c]; }
}

}  // extern "C"
