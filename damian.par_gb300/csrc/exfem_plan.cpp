// exfem_plan.cpp — host-side preparation of the device model (see exfem_plan.h).
#include "exfem_plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace exfem {

namespace {
constexpr double U_PI = 3.14159265358979323846;
constexpr double U_TOL = 1.0e-9;
const double F_WANGZERO = (double)0.0001f;   // pwaves.f90:8 (single literal in a real*8)
inline bool realunder(double a, double b) { return (a - b) < -U_TOL; }
inline bool realover(double a, double b) { return (a - b) > U_TOL; }

// 21 bits to the even bit positions 0, 2, ..., 40 (a 2-D Morton interleave).
uint64_t spread2(uint64_t v) {
    v &= 0x1fffff;
    v = (v | v << 16) & 0x001f0000ffffULL;
    v = (v | v << 8) & 0x001f00ff00ffULL;
    v = (v | v << 4) & 0x010f0f0f0f0fULL;
    v = (v | v << 2) & 0x013333333333ULL;
    v = (v | v << 1) & 0x015555555555ULL;
    return v;
}

struct Morton {
    double x0, y0, sx, sy;
    Morton(const double *xs, const double *ys, long long n) {
        double xmin = 1e300, xmax = -1e300, ymin = 1e300, ymax = -1e300;
#pragma omp parallel for schedule(static) reduction(min : xmin, ymin) reduction(max : xmax, ymax)
        for (long long i = 0; i < n; ++i) {
            xmin = std::min(xmin, xs[i]); xmax = std::max(xmax, xs[i]);
            ymin = std::min(ymin, ys[i]); ymax = std::max(ymax, ys[i]);
        }
        x0 = xmin; y0 = ymin;
        double span = std::max(std::max(xmax - xmin, ymax - ymin), 1e-30);
        sx = sy = 2097151.0 / span;
    }
    uint64_t key(double x, double y) const {
        uint64_t ix = (uint64_t)std::llround((x - x0) * sx), iy = (uint64_t)std::llround((y - y0) * sy);
        // y bit b above x bit b above y bit b - 1: keys below 2^42
        return spread2(ix) | (spread2(iy) << 1);
    }
};
}  // namespace

// initplanewaves (pwaves.f90:16-98), kept in the order of the reference's
// arithmetic; EXFEM_E_UNSUPPORTED where the reference exits.
int init_wave_const(const exfem_wave &w, double alpha, double beta, WaveConst &o, std::string &err) {
    o = WaveConst();
    o.kind = w.kind;
    o.alpha = alpha;
    o.beta = beta;
    o.freq = w.freq;
    o.fp = w.freq * U_PI;
    o.t0 = w.t0;
    if (!(alpha > 0) || !(beta > 0) || !(w.freq > 0) || !std::isfinite(w.angle) || !std::isfinite(w.amp)) {
        err = "wave parameters must be finite with positive velocities and frequency";
        return EXFEM_E_ARG;
    }
    double wa = 0, wb = 0;
    if (w.kind == EXFEM_WAVE_P) {
        double e = w.angle, a = w.amp;
        o.sine = std::sin(e);
        o.sinf = o.sine * (beta / alpha);
        double f = std::asin(o.sinf);
        o.cose = std::cos(e);
        o.cosf = std::cos(f);
        if (o.cose < F_WANGZERO) {
            err = "P wave at grazing incidence is not supported (pwaves.f90:32-35)";
            return EXFEM_E_UNSUPPORTED;
        } else if (std::fabs(o.sine) < F_WANGZERO) {
            wa = a; o.wa1 = -wa; o.wb1 = 0.0; o.cose = 1; o.sine = 0;
        } else {
            double sin2e = std::sin(2 * e), sin2f = std::sin(2 * f), cos2f = std::cos(2 * f), r = alpha / beta;
            wa = a;
            o.wa1 = (sin2e * sin2f - (r * r) * (cos2f * cos2f));
            o.wa1 = o.wa1 / (sin2e * sin2f + (r * r) * (cos2f * cos2f));
            o.wa1 = o.wa1 * a;
            o.wb1 = -(2 * r * sin2e * cos2f);
            o.wb1 = o.wb1 / (sin2e * sin2f + (r * r) * (cos2f * cos2f));
            o.wb1 = o.wb1 * a;
        }
        o.amp0 = wa;
        o.wui[0] = o.sine; o.wui[1] = -o.cose;
        o.wui[2] = o.sine; o.wui[3] = o.cose;
        o.wui[4] = -o.cosf; o.wui[5] = o.sinf;
    } else if (w.kind == EXFEM_WAVE_SV) {
        double f = w.angle, b = w.amp;
        o.sinf = std::sin(f);
        double fcr = std::asin(beta / alpha);
        o.sine = o.sinf * (alpha / beta);
        double e = std::asin(o.sine);
        o.cose = std::cos(e);
        o.cosf = std::cos(f);
        if (std::fabs(o.sinf) < F_WANGZERO) {
            wb = b; o.wb1 = -wb; o.wa1 = 0.0; o.cosf = 1; o.sinf = 0;
        } else if ((fcr - f) > F_WANGZERO) {
            double sin2e = std::sin(2 * e), sin2f = std::sin(2 * f), cos2f = std::cos(2 * f), r = alpha / beta;
            wb = b;
            o.wb1 = (sin2e * sin2f - (r * r) * (cos2f * cos2f));
            o.wb1 = o.wb1 / (sin2e * sin2f + (r * r) * (cos2f * cos2f));
            o.wb1 = o.wb1 * b;
            o.wa1 = r * std::sin(4.0 * f);
            o.wa1 = o.wa1 / (sin2e * sin2f + (r * r) * (cos2f * cos2f));
            o.wa1 = o.wa1 * b;
        } else {
            err = "SV wave at or beyond the critical angle asin(vs/vp) is not supported (pwaves.f90:87-89)";
            return EXFEM_E_UNSUPPORTED;
        }
        o.amp0 = wb;
        o.wui[0] = o.cosf; o.wui[1] = o.sinf;
        o.wui[2] = o.sine; o.wui[3] = o.cose;
        o.wui[4] = -o.cosf; o.wui[5] = o.sinf;
    } else {
        err = "wave kind must be EXFEM_WAVE_P or EXFEM_WAVE_SV";
        return EXFEM_E_ARG;
    }
    return EXFEM_OK;
}

// Inclusive prefix sum in place over a[0..n).  Two passes over fixed chunks:
// integer sums, so the result is exact whatever the thread count.
static void scan_inclusive(int *a, long long n) {
    constexpr int NCH = 64;
    if (n < (1 << 16)) {
        for (long long i = 1; i < n; ++i) a[i] += a[i - 1];
        return;
    }
    const long long chunk = (n + NCH - 1) / NCH;
    long long part[NCH + 1] = {0};
#pragma omp parallel for schedule(static, 1)
    for (int t = 0; t < NCH; ++t) {
        const long long lo = t * chunk, hi = std::min(n, lo + chunk);
        long long s = 0;
        for (long long i = lo; i < hi; ++i) s += a[i];
        part[t + 1] = s;
    }
    for (int t = 0; t < NCH; ++t) part[t + 1] += part[t];
#pragma omp parallel for schedule(static, 1)
    for (int t = 0; t < NCH; ++t) {
        const long long lo = t * chunk, hi = std::min(n, lo + chunk);
        int s = (int)part[t];
        for (long long i = lo; i < hi; ++i) {
            s += a[i];
            a[i] = s;
        }
    }
}

// CSR pointers from per-row counts: ptr[0] = 0 and ptr[i + 1] holds row i's
// count on entry, the row start sums on return.
static void counts_to_ptr(pvec<int> &ptr) {
    ptr[0] = 0;
    if (ptr.size() > 1) scan_inclusive(ptr.data() + 1, (long long)ptr.size() - 1);
}

// The ids i in [0, n) with keep(i) true, in increasing order (parallel
// stream compaction over fixed chunks).
template <class F>
static void compact_ids(int n, F keep, pvec<int> &out) {
    constexpr int NCH = 64;
    const int chunk = (n + NCH - 1) / NCH;
    int part[NCH + 1] = {0};
#pragma omp parallel for schedule(static, 1)
    for (int t = 0; t < NCH; ++t) {
        const int lo = std::min(n, t * chunk), hi = std::min(n, lo + chunk);
        int c = 0;
        for (int i = lo; i < hi; ++i) c += keep(i) ? 1 : 0;
        part[t + 1] = c;
    }
    for (int t = 0; t < NCH; ++t) part[t + 1] += part[t];
    out.resize(part[NCH]);
#pragma omp parallel for schedule(static, 1)
    for (int t = 0; t < NCH; ++t) {
        const int lo = std::min(n, t * chunk), hi = std::min(n, lo + chunk);
        int o = part[t];
        for (int i = lo; i < hi; ++i)
            if (keep(i)) out[o++] = i;
    }
}

// Stable LSD radix sort of the ids idx[0..n) by key[id]: 11-bit digits, so a
// pass's 2048 scatter streams stay in cache; a pass whose digit is the same
// for every key is skipped.  Each pass splits the array into chunks that count
// (into a local histogram) and scatter in parallel; the offsets are laid out
// digit-major then chunk-major, so the result is the stable order whatever
// the chunk or thread count.  Sorts contiguous (key, id) records so every pass
// streams through memory.
struct KeyId {
    uint64_t key;
    int id;
};
// The same order from 8-byte records: a key below 2^42 and an id below 2^22
// packed as key << 22 | id, sorted on the key bits only.  The ids start
// increasing (the callers' initial orders), so the stable passes leave equal
// keys in id order, as the 16-byte form does; half the bytes per pass.
static void radix_order_packed(const uint64_t *key, int *idx, long long n) {
    constexpr int BITS = 11;
    constexpr int NB = 1 << BITS;
    constexpr int IDB = 22;
    const int nch = (int)std::min<long long>(64, std::max<long long>(1, n / 16384));
    const long long chunk = (n + nch - 1) / nch;
    pvec<uint64_t> a, b;
    a.resize(n);
    b.resize(n);
    uint64_t any = 0, all = ~0ull;
#pragma omp parallel for schedule(static) reduction(| : any) reduction(& : all)
    for (long long i = 0; i < n; ++i) {
        a[i] = (key[idx[i]] << IDB) | (uint64_t)idx[i];
        any |= a[i];
        all &= a[i];
    }
    std::vector<long long> off((size_t)NB * nch);
    for (int sh = IDB; sh < 64; sh += BITS) {
        if ((((any ^ all) >> sh) & (NB - 1)) == 0) continue;
#pragma omp parallel for schedule(static, 1)
        for (int t = 0; t < nch; ++t) {
            long long h[NB] = {0};
            const long long lo = t * chunk, hi = std::min(n, lo + chunk);
            for (long long i = lo; i < hi; ++i) h[(a[i] >> sh) & (NB - 1)]++;
            for (int d = 0; d < NB; ++d) off[(size_t)d * nch + t] = h[d];
        }
        long long run = 0;
        for (size_t i = 0; i < off.size(); ++i) {
            const long long c = off[i];
            off[i] = run;
            run += c;
        }
#pragma omp parallel for schedule(static, 1)
        for (int t = 0; t < nch; ++t) {
            long long h[NB];
            for (int d = 0; d < NB; ++d) h[d] = off[(size_t)d * nch + t];
            const long long lo = t * chunk, hi = std::min(n, lo + chunk);
            for (long long i = lo; i < hi; ++i) b[h[(a[i] >> sh) & (NB - 1)]++] = a[i];
        }
        a.swap(b);
    }
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) idx[i] = (int)(a[i] & ((1ull << IDB) - 1));
}

static void radix_order(const uint64_t *key, int *idx, long long n, long long id_bound) {
    if (n < 2) return;
    // Morton keys are 42 bits: ids below 2^22 pack beside them
    if (id_bound <= (1LL << 22)) {
        radix_order_packed(key, idx, n);
        return;
    }
    constexpr int BITS = 11;
    constexpr int NB = 1 << BITS;
    const int nch = (int)std::min<long long>(64, std::max<long long>(1, n / 16384));   // chunks per pass
    const long long chunk = (n + nch - 1) / nch;
    pvec<KeyId> a, b;
    a.resize(n);
    b.resize(n);
    uint64_t any = 0, all = ~0ull;
#pragma omp parallel for schedule(static) reduction(| : any) reduction(& : all)
    for (long long i = 0; i < n; ++i) {
        a[i] = {key[idx[i]], idx[i]};
        any |= a[i].key;
        all &= a[i].key;
    }
    std::vector<long long> off((size_t)NB * nch);   // [digit][chunk]
    for (int sh = 0; sh < 64; sh += BITS) {
        if ((((any ^ all) >> sh) & (NB - 1)) == 0) continue;
#pragma omp parallel for schedule(static, 1)
        for (int t = 0; t < nch; ++t) {
            long long h[NB] = {0};
            const long long lo = t * chunk, hi = std::min(n, lo + chunk);
            for (long long i = lo; i < hi; ++i) h[(a[i].key >> sh) & (NB - 1)]++;
            for (int d = 0; d < NB; ++d) off[(size_t)d * nch + t] = h[d];
        }
        long long run = 0;
        for (size_t i = 0; i < off.size(); ++i) {
            const long long c = off[i];
            off[i] = run;
            run += c;
        }
#pragma omp parallel for schedule(static, 1)
        for (int t = 0; t < nch; ++t) {
            long long h[NB];
            for (int d = 0; d < NB; ++d) h[d] = off[(size_t)d * nch + t];
            const long long lo = t * chunk, hi = std::min(n, lo + chunk);
            for (long long i = lo; i < hi; ++i) b[h[(a[i].key >> sh) & (NB - 1)]++] = a[i];
        }
        a.swap(b);
    }
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) idx[i] = a[i].id;
}

int build_plan(const exfem_mesh &mesh, const exfem_problem &prob, bool reorder, Plan &P, std::string &err,
               int r_internal, bool fp64_operator) {
    const int nn = mesh.nnodes, ne = mesh.nelems;
    if (nn <= 0 || ne <= 0 || !mesh.eptr || !mesh.eind || !mesh.ediv || !mesh.nodes || !mesh.ematprop) {
        err = "mesh arrays missing or empty";
        return EXFEM_E_ARG;
    }
    if (prob.nmat <= 0 || !prob.matconst || !prob.absorbing || prob.nrhs <= 0 || (!prob.waves && prob.nseismic > 0)) {
        err = "problem arrays missing (matconst/absorbing, or waves with a DRM layer)";
        return EXFEM_E_ARG;
    }
    if (prob.point_kind != 0 && prob.point_kind != EXFEM_POINT_FORCE && prob.point_kind != EXFEM_POINT_DISP) {
        err = "unknown point source kind";
        return EXFEM_E_ARG;
    }
    if (prob.point_kind != 0 &&
        (prob.npoint < 0 || (prob.npoint > 0 && !prob.point_nodes) || !(prob.point_sigma > 0) ||
         !std::isfinite(prob.point_amp) || !std::isfinite(prob.point_t0))) {
        err = "point source needs npoint >= 0 node ids, sigma > 0 and finite amplitude and start";
        return EXFEM_E_ARG;
    }
    if (!(prob.deltat > 0) || prob.nsteps < 0 || prob.io_interval < 1) {
        err = "deltat must be > 0, nsteps >= 0 and io_interval >= 1";
        return EXFEM_E_ARG;
    }
    if (prob.nhanging < 0 || prob.nseismic < 0 || prob.nrecv < 0 ||
        (prob.nhanging > 0 && !prob.hanging) || (prob.nseismic > 0 && !prob.seismic) ||
        (prob.nrecv > 0 && (!prob.recv_xy || !prob.recv_elem))) {
        err = "hanging/seismic/receiver arrays inconsistent with their counts";
        return EXFEM_E_ARG;
    }
    if ((long long)ne * 8 >= (1LL << 30) || nn >= (1 << 29)) {
        err = "mesh too large for 32-bit gather entries";
        return EXFEM_E_ARG;
    }
    P.nn = nn; P.ne = ne; P.R_user = prob.nrhs; P.R = std::max(prob.nrhs, r_internal);
    P.dt = prob.deltat;
    // setupconstants (explicit.f90:72-77)
    P.a1 = 1.0 / (P.dt * P.dt);
    P.a2 = 1.0 / (2.0 * P.dt);
    P.a3 = 2.0 * P.a1;
    P.nsteps = prob.nsteps;
    P.io = prob.io_interval;
    P.nsave = prob.nsteps / prob.io_interval + 1;
    P.worigin[0] = prob.worigin[0];
    P.worigin[1] = prob.worigin[1];

    // ---- corners (elemallnhnodes, model.f90:163-174) and validation.  The
    // checks run in parallel; the first failing element (lowest id) is then
    // checked again alone for its message.
    if (mesh.eptr[0] != 1) { err = "eptr[0] must be 1 (1-based CSR)"; return EXFEM_E_MESH; }
    pvec<int> corner_ref;
    corner_ref.resize((size_t)ne * 4);
    auto check_elem = [&](int e, std::string *msg) -> bool {
        const int b = mesh.eptr[e] - 1, t = mesh.eptr[e + 1] - 1;
        if (t <= b || t - b > 8) {
            if (msg) *msg = "element " + std::to_string(e + 1) + " has a bad CSR row";
            return false;
        }
        int k = 0;
        for (int j = b; j < t; ++j) {
            const int v = mesh.eind[j];
            if (v < 1 || v > nn) {
                if (msg) *msg = "eind out of range in element " + std::to_string(e + 1);
                return false;
            }
            if (!mesh.ediv[j]) {
                if (k < 4) corner_ref[(size_t)e * 4 + k] = v - 1;
                ++k;
            }
        }
        if (k != 4) {
            if (msg)
                *msg = "element " + std::to_string(e + 1) + " has " + std::to_string(k) +
                       " non-hanging nodes (model.f90:166-171)";
            return false;
        }
        const int m = mesh.ematprop[e];
        if (m < 1 || m > prob.nmat) {
            if (msg) *msg = "ematprop out of range in element " + std::to_string(e + 1);
            return false;
        }
        return true;
    };
    {
        int first_bad = ne;
#pragma omp parallel for schedule(static) reduction(min : first_bad)
        for (int e = 0; e < ne; ++e)
            if (!check_elem(e, nullptr)) first_bad = std::min(first_bad, e);
        if (first_bad < ne) {
            check_elem(first_bad, &err);
            return EXFEM_E_MESH;
        }
    }
    // ---- hanging entries
    std::vector<int> hang_of(nn, -1);   // reference node -> hanging entry
    for (int i = 0; i < prob.nhanging; ++i) {
        int h = prob.hanging[3 * i] - 1, a = prob.hanging[3 * i + 1] - 1, b = prob.hanging[3 * i + 2] - 1;
        if (h < 0 || h >= nn || a < 0 || a >= nn || b < 0 || b >= nn || h == a || h == b) {
            err = "hanging entry " + std::to_string(i + 1) + " out of range";
            return EXFEM_E_MESH;
        }
        if (hang_of[h] >= 0) { err = "node " + std::to_string(h + 1) + " listed twice as hanging"; return EXFEM_E_MESH; }
        hang_of[h] = i;
    }
    for (int i = 0; i < prob.nhanging; ++i) {
        int a = prob.hanging[3 * i + 1] - 1, b = prob.hanging[3 * i + 2] - 1;
        if (hang_of[a] >= 0 || hang_of[b] >= 0) {
            // a 2:1-balanced quadtree (mesh_utils.f90:124-135) never anchors a
            // hanging node on another hanging node
            err = "chained hanging nodes (an anchor is itself hanging) are not supported";
            return EXFEM_E_UNSUPPORTED;
        }
    }
    // ---- internal numbering (Morton order; active nodes first, hanging last)
    pvec<double> xs, ys;
    xs.resize(nn);
    ys.resize(nn);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nn; ++i) { xs[i] = mesh.nodes[2 * i]; ys[i] = mesh.nodes[2 * i + 1]; }
    // active nodes in Morton order (stable), then hanging entry i as node n_active + i
    P.n_hang = prob.nhanging;
    P.n_active = nn - P.n_hang;
    pvec<int> &order = P.ref_of_node;
    order.reserve(nn);
    compact_ids(nn, [&](int i) { return hang_of[i] < 0; }, order);
    Morton mort(xs.data(), ys.data(), nn);
    if (reorder) {
        pvec<uint64_t> keys;
        keys.resize(nn);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nn; ++i) keys[i] = mort.key(xs[i], ys[i]);
        radix_order(keys.data(), order.data(), (long long)order.size(), nn);
    }
    order.resize(nn);
    for (int i = 0; i < prob.nhanging; ++i) order[(size_t)P.n_active + i] = prob.hanging[3 * i] - 1;
    // every reference node appears once in order: the scatter sets each entry
    P.node_of_ref.resize(nn);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nn; ++i) P.node_of_ref[order[i]] = i;

    pvec<int> &eorder = P.ref_of_elem;
    eorder.resize(ne);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < ne; ++e) eorder[e] = e;
    if (reorder) {
        pvec<uint64_t> ek;
        ek.resize(ne);
#pragma omp parallel for schedule(static)
        for (int e = 0; e < ne; ++e) {
            const int *c = &corner_ref[(size_t)e * 4];
            double cx = 0.25 * (xs[c[0]] + xs[c[1]] + xs[c[2]] + xs[c[3]]);
            double cy = 0.25 * (ys[c[0]] + ys[c[1]] + ys[c[2]] + ys[c[3]]);
            ek[e] = mort.key(cx, cy);
        }
        radix_order(ek.data(), eorder.data(), ne, ne);
    }
    pvec<int> &elem_of_ref = P.elem_of_ref;   // kept for point sampling
    elem_of_ref.resize(ne);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < ne; ++e) elem_of_ref[eorder[e]] = e;

    // ---- per-element data (internal order); dashpot slots numbered in that order
    P.econn.resize((size_t)ne * 4);
    P.ecoef32.resize((size_t)ne * 4);
    P.ecoef2.resize((size_t)ne * 2);
    P.emass.resize(ne);
    if (fp64_operator) {
        P.ecoef.resize((size_t)ne * 4);
        P.emulam.resize((size_t)ne * 2);
        P.ekv.resize((size_t)ne * 6);
    } else {
        P.ecoef.clear();
        P.emulam.clear();
        P.ekv.clear();
    }
    P.edampv.clear();
    pvec<double> eh;
    eh.resize(ne);
    pvec<char> damped;
    damped.resize(ne);
    int bad_elem = ne;   // first element (reference id) with a bad length or density
#pragma omp parallel for schedule(static) reduction(min : bad_elem)
    for (int ie = 0; ie < ne; ++ie) {
        int e = eorder[ie];
        const int *c = &corner_ref[(size_t)e * 4];
        for (int k = 0; k < 4; ++k) P.econn[(size_t)ie * 4 + k] = P.node_of_ref[c[k]];
        const double *mc = &prob.matconst[5 * (mesh.ematprop[e] - 1)];
        double mu = mc[0], lam = mc[1], rho = mc[2];
        double h = ys[c[2]] - ys[c[0]];   // elength (model.f90:112-118)
        damped[ie] = 0;
        if (!(h > 0) || !(rho > 0)) { bad_elem = std::min(bad_elem, e); continue; }
        eh[ie] = h;
        // the closed form's coefficients in FP64, and the FP32 form's two
        // stored values and the four it derives from them (fp32_coef)
        const double co[4] = {(lam + 2.0 * mu) / 4.0, lam / 4.0, mu / 4.0, (lam + 3.0 * mu) / 12.0};
        P.ecoef2[(size_t)ie * 2] = (float)(lam / 12.0);
        P.ecoef2[(size_t)ie * 2 + 1] = (float)(mu / 4.0);
        fp32_coef(P.ecoef2[(size_t)ie * 2], P.ecoef2[(size_t)ie * 2 + 1], &P.ecoef32[(size_t)ie * 4]);
        if (fp64_operator) {
            P.emulam[(size_t)ie * 2] = mu;
            P.emulam[(size_t)ie * 2 + 1] = lam;
            calck_values(mu, lam, &P.ekv[(size_t)ie * 6]);
            for (int k = 0; k < 4; ++k) P.ecoef[(size_t)ie * 4 + k] = co[k];
        }
        double scl = h / 2.0;
        P.emass[ie] = (scl * scl) * rho;   // calcm (formulation.f90:250-254)
        for (int k = 0; k < 4; ++k) {
            int ab = prob.absorbing[c[k]];
            if (ab == 1 || ab == 2) damped[ie] = 1;
        }
    }
    if (bad_elem < ne) {
        err = "element " + std::to_string(bad_elem + 1) + " has non-positive length or density";
        return EXFEM_E_MESH;
    }
    {
        // dashpot slot of element ie: the damped elements before it
        P.edamp.resize(ne);
#pragma omp parallel for schedule(static)
        for (int ie = 0; ie < ne; ++ie) P.edamp[ie] = damped[ie];
        scan_inclusive(P.edamp.data(), ne);
        const int nd = P.edamp[ne - 1];
#pragma omp parallel for schedule(static)
        for (int ie = 0; ie < ne; ++ie) P.edamp[ie] = damped[ie] ? P.edamp[ie] - 1 : -1;
        P.edampv.assign((size_t)nd * 8, 0.0);
#pragma omp parallel for schedule(static)
        for (int ie = 0; ie < ne; ++ie) {
            if (!damped[ie]) continue;
            int e = eorder[ie];
            const int *c = &corner_ref[(size_t)e * 4];
            const double *mc = &prob.matconst[5 * (mesh.ematprop[e] - 1)];
            const double rho = mc[2], vp = mc[3], vs = mc[4], h = eh[ie];
            double *damping = &P.edampv[(size_t)P.edamp[ie] * 8];
            for (int k = 0; k < 4; ++k) {   // getdampingof + lysmer (model.f90:585-604)
                int ab = prob.absorbing[c[k]];
                if (ab == 1 || ab == 2) {
                    double r0 = vp * rho * h, r1 = vs * rho * h;
                    if (ab == 1) { damping[2 * k] = r1; damping[2 * k + 1] = r0; }
                    else { damping[2 * k] = r0; damping[2 * k + 1] = r1; }
                }
            }
        }
    }
    // ---- own incidences per node (internal ids) in reference element order:
    // counted and placed in parallel, then each node's few entries are sorted
    // by (reference element, corner), the order the element loop adds them
    const long long ncorn = 4LL * ne;
    P.ownptr.resize((size_t)nn + 1);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i <= nn; ++i) P.ownptr[i] = 0;
#pragma omp parallel for schedule(static)
    for (long long j = 0; j < ncorn; ++j) __atomic_fetch_add(&P.ownptr[(size_t)P.econn[j] + 1], 1, __ATOMIC_RELAXED);
    counts_to_ptr(P.ownptr);
    P.ownlist.resize(P.ownptr[nn]);
    {
        pvec<int> fill;
        fill.resize(nn);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nn; ++i) fill[i] = P.ownptr[i];
#pragma omp parallel for schedule(static)
        for (long long j = 0; j < ncorn; ++j) {
            const int s = __atomic_fetch_add(&fill[P.econn[j]], 1, __ATOMIC_RELAXED);
            P.ownlist[s] = (int)j;
        }
        auto order_key = [&](int v) { return eorder[v >> 2] * 4 + (v & 3); };
#pragma omp parallel for schedule(static)
        for (int x = 0; x < nn; ++x) {
            int *l = &P.ownlist[P.ownptr[x]];
            const int cnt = P.ownptr[x + 1] - P.ownptr[x];
            for (int i = 1; i < cnt; ++i) {
                const int v = l[i], kv = order_key(v);
                int j = i - 1;
                while (j >= 0 && order_key(l[j]) > kv) { l[j + 1] = l[j]; --j; }
                l[j + 1] = v;
            }
        }
    }
    {
        int first_lonely = nn;
#pragma omp parallel for schedule(static) reduction(min : first_lonely)
        for (int i = 0; i < nn; ++i)
            if (P.ownptr[i + 1] == P.ownptr[i]) first_lonely = std::min(first_lonely, i);
        if (first_lonely < nn) {
            err = "node " + std::to_string(P.ref_of_node[first_lonely] + 1) + " is not a non-hanging corner of any element";
            return EXFEM_E_MESH;
        }
    }
    // ---- m_full (init_explicit, explicit.f90:95-106): each dof sums its
    // element terms in reference element order (the incidence lists' order),
    // as the element loop adds them; then sum_reactanchors in halving form.
    // ref_of_node is a permutation, so the loop sets every entry.
    P.mfull_ref.resize((size_t)2 * nn);
#pragma omp parallel for schedule(static)
    for (int n = 0; n < nn; ++n) {
        const size_t x = (size_t)P.ref_of_node[n];
        double acc[2] = {0.0, 0.0};
        for (int q = P.ownptr[n]; q < P.ownptr[n + 1]; ++q) {
            const int ie = P.ownlist[q] >> 2, k = P.ownlist[q] & 3;
            const double mass = P.emass[ie];
            const double *dv = P.edamp[ie] >= 0 ? &P.edampv[(size_t)P.edamp[ie] * 8] : nullptr;
            for (int d = 0; d < 2; ++d) {
                double damping = dv ? dv[2 * k + d] : 0.0;
                // e_mfull(dofs) + e_a(2)*damping + e_a(1)*mass, left to right
                acc[d] = (acc[d] + P.a2 * damping) + P.a1 * mass;
            }
        }
        P.mfull_ref[2 * x] = acc[0];
        P.mfull_ref[2 * x + 1] = acc[1];
    }
    for (int i = 0; i < prob.nhanging; ++i) {   // sum_reactanchors, halving form
        int h = prob.hanging[3 * i] - 1, a = prob.hanging[3 * i + 1] - 1, b = prob.hanging[3 * i + 2] - 1;
        for (int k = 0; k < 2; ++k) {
            double red = P.mfull_ref[2 * h + k] / 2.0;
            P.mfull_ref[2 * a + k] += red;
            P.mfull_ref[2 * b + k] += red;
        }
    }
    P.inv_mfull.resize((size_t)2 * P.n_active);
    P.mfull_int.resize((size_t)2 * P.n_active);
    {
        int first_bad = P.n_active;
#pragma omp parallel for schedule(static) reduction(min : first_bad)
        for (int n = 0; n < P.n_active; ++n)
            for (int k = 0; k < 2; ++k) {
                double m = P.mfull_ref[(size_t)P.ref_of_node[n] * 2 + k];
                if (!(m > 0)) first_bad = std::min(first_bad, n);
                P.inv_mfull[(size_t)2 * n + k] = 1.0 / m;
                P.mfull_int[(size_t)2 * n + k] = m;
            }
        if (first_bad < P.n_active) {
            err = "non-positive lumped mass at node " + std::to_string(P.ref_of_node[first_bad] + 1);
            return EXFEM_E_MESH;
        }
    }
    // ---- hanging entries (internal) and per-anchor links (h, other anchor), entry order
    P.hang.resize((size_t)3 * P.n_hang);
    P.lptr.resize((size_t)P.n_active + 1);
#pragma omp parallel for schedule(static)
    for (int n = 0; n <= P.n_active; ++n) P.lptr[n] = 0;
    for (int i = 0; i < prob.nhanging; ++i) {
        int h = P.node_of_ref[prob.hanging[3 * i] - 1];
        int a = P.node_of_ref[prob.hanging[3 * i + 1] - 1];
        int b = P.node_of_ref[prob.hanging[3 * i + 2] - 1];
        P.hang[3 * (size_t)i] = h; P.hang[3 * (size_t)i + 1] = a; P.hang[3 * (size_t)i + 2] = b;
        P.lptr[a + 1]++;
        P.lptr[b + 1]++;
    }
    counts_to_ptr(P.lptr);
    P.llist.assign(2 * (size_t)P.lptr[P.n_active], 0);
    if (prob.nhanging > 0) {
        pvec<int> fill;
        fill.resize(P.n_active);
#pragma omp parallel for schedule(static)
        for (int n = 0; n < P.n_active; ++n) fill[n] = P.lptr[n];
        for (int i = 0; i < prob.nhanging; ++i) {
            int h = P.hang[3 * (size_t)i], a = P.hang[3 * (size_t)i + 1], b = P.hang[3 * (size_t)i + 2];
            int qa = fill[a]++, qb = fill[b]++;
            P.llist[2 * (size_t)qa] = h; P.llist[2 * (size_t)qa + 1] = b;
            P.llist[2 * (size_t)qb] = h; P.llist[2 * (size_t)qb + 1] = a;
        }
    }
    // ---- gather lists of active nodes: own terms, then linked hanging terms at 1/2
    P.tptr.resize((size_t)P.n_active + 1);
#pragma omp parallel for schedule(static)
    for (int n = 0; n < P.n_active; ++n) {
        int cnt = P.ownptr[n + 1] - P.ownptr[n];
        for (int q = P.lptr[n]; q < P.lptr[n + 1]; ++q) {
            int h = P.llist[2 * (size_t)q];
            cnt += P.ownptr[h + 1] - P.ownptr[h];
        }
        P.tptr[n + 1] = cnt;
    }
    counts_to_ptr(P.tptr);
    P.tlist.resize(P.tptr[P.n_active]);
#pragma omp parallel for schedule(static)
    for (int n = 0; n < P.n_active; ++n) {
        int o = P.tptr[n];
        for (int q = P.ownptr[n]; q < P.ownptr[n + 1]; ++q) P.tlist[o++] = P.ownlist[q] << 1;
        for (int l = P.lptr[n]; l < P.lptr[n + 1]; ++l) {
            int h = P.llist[2 * (size_t)l];
            for (int q = P.ownptr[h]; q < P.ownptr[h + 1]; ++q) P.tlist[o++] = (P.ownlist[q] << 1) | 1;
        }
    }
    // ---- per-node lumped mass / damping (internal), for the FP32 increment form
    P.nmass.resize(nn);
    P.ndamp.resize((size_t)2 * nn);
#pragma omp parallel for schedule(static)
    for (int x = 0; x < nn; ++x) {
        double ms = 0.0, d0 = 0.0, d1 = 0.0;
        for (int q = P.ownptr[x]; q < P.ownptr[x + 1]; ++q) {
            const int ie = P.ownlist[q] >> 2, k = P.ownlist[q] & 3;
            ms += P.emass[ie];
            if (P.edamp[ie] >= 0) {
                const double *dv = &P.edampv[(size_t)P.edamp[ie] * 8];
                d0 += dv[2 * k];
                d1 += dv[2 * k + 1];
            }
        }
        P.nmass[x] = ms;
        P.ndamp[2 * (size_t)x] = d0;
        P.ndamp[2 * (size_t)x + 1] = d1;
    }
    // ---- DRM slots (wave_elems output, model.f90:1015-1045)
    P.s_elem.resize(prob.nseismic);
    P.s_kind.resize(prob.nseismic);
    std::vector<std::pair<int, int>> dent;   // (active node, entry) in slot order
    for (int s = 0; s < prob.nseismic; ++s) {
        int e = prob.seismic[2 * s] - 1, kind = prob.seismic[2 * s + 1];
        if (e < 0 || e >= ne || !(kind == 1 || kind == 2 || kind == 4 || kind == 5 || kind == 6)) {
            err = "seismic entry " + std::to_string(s + 1) + " invalid";
            return EXFEM_E_MESH;
        }
        int ie = elem_of_ref[e];
        P.s_elem[s] = ie;
        P.s_kind[s] = kind;
        for (int k = 0; k < 4; ++k) {
            int x = P.econn[(size_t)ie * 4 + k];
            int ent = (s * 4 + k) << 1;
            if (x < P.n_active) dent.push_back({x, ent});
            else {
                int hi = hang_of[P.ref_of_node[x]];
                dent.push_back({P.node_of_ref[prob.hanging[3 * hi + 1] - 1], ent | 1});
                dent.push_back({P.node_of_ref[prob.hanging[3 * hi + 2] - 1], ent | 1});
            }
        }
    }
    P.odptr.resize((size_t)nn + 1);
#pragma omp parallel for schedule(static)
    for (int i = 0; i <= nn; ++i) P.odptr[i] = 0;
    for (int s = 0; s < prob.nseismic; ++s)
        for (int k = 0; k < 4; ++k) P.odptr[P.econn[(size_t)P.s_elem[s] * 4 + k] + 1]++;
    counts_to_ptr(P.odptr);
    P.odlist.resize(P.odptr[nn]);
    if (prob.nseismic > 0) {
        pvec<int> fill;
        fill.resize(nn);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < nn; ++i) fill[i] = P.odptr[i];
        for (int s = 0; s < prob.nseismic; ++s)
            for (int k = 0; k < 4; ++k) P.odlist[fill[P.econn[(size_t)P.s_elem[s] * 4 + k]]++] = s * 4 + k;
    }
    P.dptr.resize((size_t)P.n_active + 1);
#pragma omp parallel for schedule(static)
    for (int n = 0; n <= P.n_active; ++n) P.dptr[n] = 0;
    for (auto &de : dent) P.dptr[de.first + 1]++;
    counts_to_ptr(P.dptr);
    P.dlist.resize(P.dptr[P.n_active]);
    if (!dent.empty()) {
        pvec<int> fill;
        fill.resize(P.n_active);
#pragma omp parallel for schedule(static)
        for (int n = 0; n < P.n_active; ++n) fill[n] = P.dptr[n];
        for (auto &de : dent) P.dlist[fill[de.first]++] = de.second;
    }
    // ---- kept for point sampling (elem_of_ref above): internal node coordinates
    P.nxy.resize(2 * (size_t)nn);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nn; ++i) {
        P.nxy[2 * (size_t)P.node_of_ref[i]] = xs[i];
        P.nxy[2 * (size_t)P.node_of_ref[i] + 1] = ys[i];
    }
    for (int k = 0; k < 3; ++k) P.wbox[k] = prob.wbox[k];
    P.have_waves = prob.waves != nullptr;
    // ---- receivers (visu_field, visualization.f90:156-181)
    P.nrecv = prob.nrecv;
    P.rxy.assign((size_t)2 * P.nrecv, 0.0);
    if (P.nrecv > 0) std::copy(prob.recv_xy, prob.recv_xy + 2 * (size_t)P.nrecv, P.rxy.begin());
    for (int i = 0; i < P.nrecv; ++i) {
        const int e = prob.recv_elem[i];
        if (e < 1 || e > ne) { err = "receiver " + std::to_string(i + 1) + " element out of range"; return EXFEM_E_ARG; }
    }
    if (int rc = point_weights(P, P.nrecv, prob.recv_xy, prob.recv_elem, P.rnode, P.rw, P.rsoil, err)) return rc;
    // ---- waves (none, or padding past the caller's: zero amplitudes, so their
    // free field, DRM forces and receiver samples are zero)
    P.waves.resize(P.R);
    for (int r = 0; r < P.R; ++r) {
        if (!prob.waves || r >= P.R_user) {
            P.waves[r] = WaveConst();
            P.waves[r].kind = EXFEM_WAVE_P;
            P.waves[r].alpha = P.waves[r].beta = 1.0;
            P.waves[r].cose = 1.0;
            continue;
        }
        int rc = init_wave_const(prob.waves[r], prob.walpha, prob.wbeta, P.waves[r], err);
        if (rc) { err = "rhs " + std::to_string(r) + ": " + err; return rc; }
    }
    // ---- point source: flags on internal nodes
    P.point_kind = prob.point_kind;
    P.point_amp = prob.point_amp;
    P.point_sigma = prob.point_sigma;
    P.point_t0 = prob.point_t0;
    P.pflag.assign(P.nn, 0);
    if (prob.point_kind != 0) {
        for (int i = 0; i < prob.npoint; ++i) {
            const int g = prob.point_nodes[i];
            if (g < 1 || g > nn) { err = "point source node out of range"; return EXFEM_E_ARG; }
            P.pflag[P.node_of_ref[g - 1]] = 1;
        }
    }
    return EXFEM_OK;
}

int point_weights(const Plan &P, int npt, const double *xy, const int *elem, std::vector<int> &node,
                  std::vector<double> &w, std::vector<int> &soil, std::string &err) {
    node.assign(4 * (size_t)std::max(npt, 0), -1);
    w.assign(4 * (size_t)std::max(npt, 0), 0.0);
    soil.assign(std::max(npt, 0), 0);
    for (int i = 0; i < npt; ++i) {
        const int e = elem[i];
        if (e == 0) continue;
        if (e < 1 || e > P.ne) { err = "point " + std::to_string(i + 1) + " element out of range"; return EXFEM_E_ARG; }
        const int ie = P.elem_of_ref[e - 1];
        const int *c = &P.econn[(size_t)ie * 4];
        const double px = xy[2 * (size_t)i], py = xy[2 * (size_t)i + 1];
        const double x0 = P.nxy[2 * (size_t)c[0]], y0 = P.nxy[2 * (size_t)c[0] + 1];
        const double x2 = P.nxy[2 * (size_t)c[2]], y2 = P.nxy[2 * (size_t)c[2] + 1];
        // shapeparams (formulation.f90:334-343) and shapefuncs (356-363)
        double r = (px - x0) / (x2 - x0);
        double s = (py - y0) / (y2 - y0);
        r = 2.0 * r - 1.0; s = 2.0 * s - 1.0;
        r = std::min(1.0, std::max(-1.0, r)); s = std::min(1.0, std::max(-1.0, s));
        const double inter[4] = {(1 - r) * (1 - s) / 4, (1 + r) * (1 - s) / 4, (1 + r) * (1 + s) / 4,
                                 (1 - r) * (1 + s) / 4};
        for (int k = 0; k < 4; ++k) {
            node[4 * (size_t)i + k] = c[k];
            w[4 * (size_t)i + k] = inter[k];
        }
        soil[i] = P.have_waves && (realunder(px, P.wbox[0]) || realover(px, P.wbox[1]) || realover(py, P.wbox[2]));
    }
    return EXFEM_OK;
}

int build_tiles(const Plan &P, int tn, Tiles &T, std::string &err) {
    if (tn < 1) { err = "tile size must be positive"; return EXFEM_E_ARG; }
    T = Tiles();
    T.tn = tn;
    T.ntiles = (P.n_active + tn - 1) / tn;
    T.hptr.assign(T.ntiles + 1, 0);
    T.rptr.assign(T.ntiles + 1, 0);
    T.tslot.assign(4 * P.tlist.size(), 0);
    T.nslot.assign(P.n_active, 0);
    T.lslot.assign(P.llist.size() / 2, 0);
    std::vector<int> slot(P.nn, -1), nodes;
    for (int t = 0; t < T.ntiles; ++t) {
        int n0 = t * tn, n1 = std::min(P.n_active, n0 + tn);
        nodes.clear();
        for (int n = n0; n < n1; ++n) {
            nodes.push_back(n);
            for (int q = P.tptr[n]; q < P.tptr[n + 1]; ++q) {
                int e = (P.tlist[q] >> 1) >> 2;
                for (int v = 0; v < 4; ++v) nodes.push_back(P.econn[(size_t)e * 4 + v]);
            }
            for (int q = P.lptr[n]; q < P.lptr[n + 1]; ++q) nodes.push_back(P.llist[2 * (size_t)q]);
        }
        std::sort(nodes.begin(), nodes.end());
        nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
        if (nodes.size() > 65535) { err = "tile halo too large"; return EXFEM_E_ARG; }
        for (size_t i = 0; i < nodes.size(); ++i) slot[nodes[i]] = (int)i;
        T.hlist.insert(T.hlist.end(), nodes.begin(), nodes.end());
        T.hptr[t + 1] = (int)T.hlist.size();
        for (size_t i = 0; i < nodes.size();) {
            size_t j = i + 1;
            while (j < nodes.size() && nodes[j] == nodes[j - 1] + 1) ++j;
            T.runs.push_back(nodes[i]);
            T.runs.push_back((int)(j - i));
            i = j;
        }
        T.rptr[t + 1] = (int)(T.runs.size() / 2);
        T.hmax = std::max(T.hmax, (int)nodes.size());
        for (int n = n0; n < n1; ++n) {
            T.nslot[n] = slot[n];
            for (int q = P.tptr[n]; q < P.tptr[n + 1]; ++q) {
                int e = (P.tlist[q] >> 1) >> 2;
                for (int v = 0; v < 4; ++v) T.tslot[4 * (size_t)q + v] = (unsigned short)slot[P.econn[(size_t)e * 4 + v]];
            }
            for (int q = P.lptr[n]; q < P.lptr[n + 1]; ++q) T.lslot[q] = slot[P.llist[2 * (size_t)q]];
        }
        for (int x : nodes) slot[x] = -1;
    }
    return EXFEM_OK;
}

bool build_mma_tiles(const Plan &P, int tn, int emax_limit, MmaTiles &T, std::string &why) {
    T = MmaTiles();
    if (tn < 1 || emax_limit < 8 || emax_limit > 255) { why = "bad tile shape"; return false; }
    T.tn = tn;
    T.tj.assign(P.tlist.size(), 0);
    T.nptr.push_back(0);
    T.eptr.push_back(0);
    std::vector<int> local(P.ne, -1), elems, fresh;
    int n = 0;
    while (n < P.n_active) {
        const int n0 = n;
        elems.clear();
        while (n < P.n_active && n - n0 < tn) {
            // the node's new elements; it joins the tile only if they fit
            fresh.clear();
            for (int q = P.tptr[n]; q < P.tptr[n + 1]; ++q) {
                const int e = (P.tlist[q] >> 1) >> 2;
                if (local[e] < 0 && std::find(fresh.begin(), fresh.end(), e) == fresh.end()) fresh.push_back(e);
            }
            if ((int)(elems.size() + fresh.size()) > emax_limit) {
                if (n == n0) {
                    why = "node " + std::to_string(n) + " reads more than " + std::to_string(emax_limit) + " elements";
                    for (int e : elems) local[e] = -1;
                    return false;
                }
                break;
            }
            for (int e : fresh) {
                local[e] = (int)elems.size();
                elems.push_back(e);
            }
            for (int q = P.tptr[n]; q < P.tptr[n + 1]; ++q) T.tj[q] = (unsigned char)local[(P.tlist[q] >> 1) >> 2];
            ++n;
        }
        T.emax = std::max(T.emax, (int)elems.size());
        T.elist.insert(T.elist.end(), elems.begin(), elems.end());
        T.eptr.push_back((int)T.elist.size());
        T.nptr.push_back(n);
        for (int e : elems) local[e] = -1;
    }
    T.ntiles = (int)T.nptr.size() - 1;
    return true;
}

pvec<float> node_coef32(const Plan &P) {
    pvec<float> nc;
    nc.resize((size_t)4 * P.n_active);
#pragma omp parallel for schedule(static)
    for (int n = 0; n < P.n_active; ++n) {
        nc[4 * (size_t)n] = (float)P.inv_mfull[2 * (size_t)n];
        nc[4 * (size_t)n + 1] = (float)P.inv_mfull[2 * (size_t)n + 1];
        nc[4 * (size_t)n + 2] = (float)(-2.0 * P.a2 * P.ndamp[2 * (size_t)n]);
        nc[4 * (size_t)n + 3] = (float)(-2.0 * P.a2 * P.ndamp[2 * (size_t)n + 1]);
    }
    return nc;
}

bool build_node_slots(const Plan &P, const pvec<float> &nc, NodeSlots &out, std::string &why) {
    out = NodeSlots();
    if ((long long)P.ne * 8 > (1ll << 31) - 1) { why = "2^28 elements or more"; return false; }
    out.slot4.resize((size_t)4 * P.n_active);
    out.invm.resize((size_t)P.n_active);
    long long marked = 0;
#pragma omp parallel for schedule(static) reduction(+ : marked)
    for (int n = 0; n < P.n_active; ++n) {
        const int q0 = P.tptr[n], nt = P.tptr[n + 1] - q0;
        int *s = &out.slot4[4 * (size_t)n];
        for (int j = 0; j < 4; ++j) s[j] = j < nt ? P.tlist[q0 + j] : -1;
        const float *c = &nc[4 * (size_t)n];
        const bool mark = nt > 4 || P.dptr[n + 1] > P.dptr[n] || P.lptr[n + 1] > P.lptr[n] || c[2] != 0.f ||
                          c[3] != 0.f || std::memcmp(&c[0], &c[1], sizeof(float)) != 0 || !(c[0] > 0.f);
        marked += mark ? 1 : 0;
        out.invm[n] = mark ? -1.f : c[0];
    }
    out.marked = marked;
    return true;
}

bool build_pipe_pack(const Plan &P, const Tiles &T, int max_runs, PipePack &out, std::string &why) {
    out = PipePack();
    if (T.hmax >= (1 << 14)) { why = "tile halo over 16383 nodes"; return false; }
    if (P.dlist.size() >= (1u << 24) || P.llist.size() / 2 >= (1u << 24)) { why = "DRM or link list over 2^24"; return false; }
    auto fbits = [](float f) { int i; std::memcpy(&i, &f, sizeof(i)); return i; };
    const pvec<float> nc = node_coef32(P);
    const int tn = T.tn;
    out.hdr.assign(4 * (size_t)T.ntiles, 0);
    out.runs.assign(2 * (size_t)max_runs * T.ntiles, 0);
    out.nrec.assign(8 * (size_t)P.n_active, 0);
    for (int t = 0; t < T.ntiles; ++t) {
        const int n0 = t * tn, n1 = std::min(P.n_active, n0 + tn);
        const int nr = T.rptr[t + 1] - T.rptr[t];
        const int q0 = P.tptr[n0], q1 = P.tptr[n1], nt = q1 - q0, ntev = (nt + 1) & ~1;
        if (nr > max_runs) { why = "tile halo in more than " + std::to_string(max_runs) + " runs"; return false; }
        if (nt >= (1 << 16)) { why = "tile with 65536 terms or more"; return false; }
        out.tmax = std::max(out.tmax, nt);
        int *h = &out.hdr[4 * (size_t)t];
        h[0] = T.hptr[t + 1] - T.hptr[t];
        h[1] = nt;
        h[2] = (int)(out.tpack.size() / 4);
        h[3] = nr;
        for (int i = 0; i < 2 * nr; ++i) out.runs[2 * (size_t)t * max_runs + i] = T.runs[2 * (size_t)T.rptr[t] + i];
        const size_t base = out.tpack.size();
        out.tpack.resize(base + 2 * (size_t)ntev + 4 * (size_t)nt, 0);
        for (int q = q0; q < q1; ++q) {
            const int ent = P.tlist[q], cor = (ent >> 1) & 3, e = (ent >> 1) >> 2;
            const float w = (ent & 1) ? 0.5f : 1.0f;
            const unsigned short *sl = &T.tslot[4 * (size_t)q];
            const unsigned s0 = (unsigned)sl[0] | ((unsigned)cor << 14);
            out.tpack[base + 2 * (size_t)(q - q0)] = (int)(s0 | ((unsigned)sl[1] << 16));
            out.tpack[base + 2 * (size_t)(q - q0) + 1] = (int)((unsigned)sl[2] | ((unsigned)sl[3] << 16));
            for (int v = 0; v < 4; ++v)
                out.tpack[base + 2 * (size_t)ntev + 4 * (size_t)(q - q0) + v] = fbits(P.ecoef32[(size_t)e * 4 + v] * w);
        }
        for (int n = n0; n < n1; ++n) {
            int *r = &out.nrec[8 * (size_t)n];
            for (int v = 0; v < 4; ++v) r[v] = fbits(nc[4 * (size_t)n + v]);
            const int tb = P.tptr[n] - q0, tc = P.tptr[n + 1] - P.tptr[n];
            const int dcnt = P.dptr[n + 1] - P.dptr[n], lcnt = P.lptr[n + 1] - P.lptr[n];
            if (dcnt > 255 || lcnt > 255) { why = "node with over 255 DRM terms or links"; return false; }
            r[4] = (int)((unsigned)tb | ((unsigned)tc << 16));
            r[5] = T.nslot[n];
            r[6] = (int)((unsigned)P.dptr[n] | ((unsigned)dcnt << 24));
            r[7] = (int)((unsigned)P.lptr[n] | ((unsigned)lcnt << 24));
        }
    }
    if (out.tpack.empty()) out.tpack.assign(4, 0);
    return true;
}

}  // namespace exfem
