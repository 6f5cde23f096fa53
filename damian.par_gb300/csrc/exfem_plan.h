// exfem_plan.h — host-side preparation of the device-resident model.
//
// Turns the reference-layout mesh/problem (include/exfem_gpu.h) into the
// arrays the kernels read: a Morton-ordered internal numbering, per-element
// Q4 operator coefficients, lumped mass/damping, the node-to-(element, corner)
// gather lists that replace the element scatter of explicit.f90:141 and the
// halo/anchor sums, the DRM slots and the receiver weights.  Pure C++ (no CUDA)
// so it can be exercised without a GPU.
#pragma once

#include <cstdint>
#include <new>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "exfem_gpu.h"

namespace exfem {

// Allocator whose no-argument construct leaves trivial elements unset, so
// resizing a large plan array does not zero it on one thread before the
// parallel loop that writes every element (first touch then happens on the
// threads that fill it).
template <class T>
struct RawAlloc : std::allocator<T> {
    template <class U>
    struct rebind { using other = RawAlloc<U>; };
    RawAlloc() = default;
    template <class U>
    RawAlloc(const RawAlloc<U> &) {}
    template <class U>
    void construct(U *p) noexcept(std::is_nothrow_default_constructible<U>::value) { ::new (static_cast<void *>(p)) U; }
    template <class U, class... A>
    void construct(U *p, A &&...a) { ::new (static_cast<void *>(p)) U(std::forward<A>(a)...); }
};
// Plan arrays: resize() leaves new elements unset; assign() and the
// initialiser forms still set them.
template <class T>
using pvec = std::vector<T, RawAlloc<T>>;

// Constants of one plane wave after initplanewaves (pwaves.f90:16-98).
struct WaveConst {
    int kind;
    double alpha, beta, freq, fp;          // fp = freq*pi
    double sine, cose, sinf, cosf;
    double amp0, wa1, wb1;                 // incident (wa or wb), reflected P, reflected SV
    double wui[6];                          // f_wui(2,3) column-major: (1,1),(2,1),(1,2),(2,2),(1,3),(2,3)
    double t0;
};

int init_wave_const(const exfem_wave &w, double alpha, double beta, WaveConst &out, std::string &err);

// The six distinct magnitudes of calck(mu, lambda) (formulation.f90:276-313),
// each with the formula's operations: (3m+l)/3, (m+l)/4, (3m+2l)/6, (m-l)/4,
// (3m+l)/6, l/6.  The FP64 kernels rebuild K from them with signs.
// The FP32 form's four closed-form coefficients ((l+2m)/4, l/4, m/4,
// (l+3m)/12) from its two stored values b3 = l/12 and c = m/4 (FP32, each
// rounded once): B = 3 b3, A = B + 2c, D = b3 + c, each an FP32 operation
// rounded once (no contraction).  The four are linear in (lambda, mu), so an
// element needs only the two values; each result is within 2 ulps of its
// FP64 value rounded once.  The device computes the same operations.
inline void fp32_coef(float b3, float c, float out[4]) {
    volatile float B = 3.0f * b3;   // separate roundings on every compiler
    volatile float c2 = 2.0f * c;
    out[1] = B;
    out[0] = B + c2;
    out[2] = c;
    out[3] = b3 + c;
}

inline void calck_values(double m, double l, double kv[6]) {
    kv[0] = (3.0 * m + l) / 3.0;
    kv[1] = (m + l) / 4.0;
    kv[2] = (3.0 * m + 2.0 * l) / 6.0;
    kv[3] = (m - l) / 4.0;
    kv[4] = (3.0 * m + l) / 6.0;
    kv[5] = l / 6.0;
}

struct Plan {
    int nn = 0, ne = 0, R = 1;
    int R_user = 1;                 // the caller's right-hand sides; R - R_user zero-amplitude padding
    int n_active = 0;               // non-hanging nodes are internal [0, n_active)
    int n_hang = 0;                 // hanging nodes are internal [n_active, nn)
    double dt = 0, a1 = 0, a2 = 0, a3 = 0;
    int nsteps = 0, io = 1, nsave = 1;
    pvec<int> ref_of_node;          // internal -> reference node (0-based)
    pvec<int> node_of_ref;          // reference -> internal
    pvec<int> ref_of_elem;          // internal -> reference element (0-based)
    // elements (internal order)
    pvec<int> econn;                // 4 per element: internal node ids of the non-hanging corners
    pvec<double> ecoef;             // 4 per element: (lam+2mu)/4, lam/4, mu/4, (lam+3mu)/12
    pvec<float> ecoef32;            // same, FP32, from ecoef2 (fp32_coef)
    pvec<float> ecoef2;             // 2 per element: lam/12 and mu/4, each rounded once to FP32
    pvec<double> emulam;            // 2 per element: (mu, lambda)
    pvec<double> ekv;               // 6 per element: calck_values(mu, lambda)
    pvec<double> emass;             // rho*(h/2)^2 per element (getmassof)
    pvec<int> edamp;                // per element: index into edampv or -1
    std::vector<double> edampv;     // 8 per damped element (getdampingof)
    // gather lists for active nodes; entry = ((elem*4 + corner) << 1) | half
    pvec<int> tptr, tlist;
    pvec<int> dptr, dlist;          // DRM: ((slot*4 + corner) << 1) | half
    pvec<double> mfull_ref;         // m_full in reference dof order (mass.bin)
    pvec<double> inv_mfull;         // 2 per active node (internal), 1/m_full
    pvec<double> mfull_int;         // 2 per active node (internal), m_full
    // per node lumped terms (internal): M_n, C_n(x,y), D_n(x,y) = a1 M + a2 C, for the FP32 form
    pvec<double> nmass, ndamp;
    // hanging entries (internal ids): h, a, b; hanging node of entry i is
    // internal node n_active + i
    std::vector<int> hang;
    // DRM (seismic) elements
    std::vector<int> s_elem, s_kind;
    // receivers: the 4 non-hanging corners (internal ids) and their shape
    // function weights (visu_field); a hanging corner is read as the average
    // of its anchors
    std::vector<int> rnode;
    std::vector<double> rw;
    std::vector<int> rsoil;
    std::vector<double> rxy;
    int nrecv = 0;
    // kept for point sampling after setup: reference -> internal element,
    // internal node coordinates, the DRM box (left, right, top)
    pvec<int> elem_of_ref;
    pvec<double> nxy;
    double wbox[3] = {0, 0, 0};
    // waves (have_waves false: zero-amplitude placeholders, no free field)
    std::vector<WaveConst> waves;
    bool have_waves = true;
    // point source (EXFEM_POINT_*): per internal node, 1 on the source nodes
    int point_kind = 0;
    double point_amp = 0, point_sigma = 1, point_t0 = 0;
    std::vector<unsigned char> pflag;
    double worigin[2] = {0, 0};
    // per active node: hanging links (h, other anchor) in m_hanging order
    pvec<int> lptr, llist;          // llist entries: h internal, b internal (pairs)
    // own incidences of every node (incl. hanging): elem*4+corner, sorted by
    // reference element index (the order explicit.f90:129-142 adds them)
    pvec<int> ownptr, ownlist;
    // own DRM incidences of every node: slot*4+corner in seismic order
    pvec<int> odptr, odlist;
};

// visu_field's interpolation data (visualization.f90:156-181) for npt points
// in 1-based reference elements: the element's 4 corners (internal ids), the
// shapefuncs weights at the clamped local coordinates (shapeparams,
// formulation.f90:315-363) and inside_soil (0 without waves).  elem 0 marks a
// point outside the mesh: corners -1, weights 0.
int point_weights(const Plan &P, int npt, const double *xy, const int *elem, std::vector<int> &node,
                  std::vector<double> &w, std::vector<int> &soil, std::string &err);

// Shared-memory tiles of the FP32 step: consecutive active nodes (Morton
// order, so a tile is a compact patch) and the halo of nodes their terms read.
struct Tiles {
    int tn = 0;                        // nodes per tile
    int ntiles = 0;
    int hmax = 0;                      // largest halo
    std::vector<int> hptr, hlist;      // halo node ids per tile (sorted)
    std::vector<unsigned short> tslot; // 4 per gather term: halo slots of the element's corners
    std::vector<int> nslot;            // per active node: its own halo slot
    std::vector<int> lslot;            // per anchor link: halo slot of the hanging node
    // runs of consecutive node ids in each tile's sorted halo (for bulk copies)
    std::vector<int> rptr;             // ntiles + 1
    std::vector<int> runs;             // (first node, count) pairs
};

int build_tiles(const Plan &P, int tn, Tiles &T, std::string &err);

// Element tiles of the tensor-core FP32 step (variant 3): runs of at most tn
// consecutive active nodes whose terms read at most emax_limit distinct
// elements (a tile closes early where the Morton order jumps between
// regions), each with its distinct elements (their K.u is computed once per
// tile), and per term the element's index in its tile's list.
struct MmaTiles {
    int tn = 0, ntiles = 0;
    int emax = 0;                      // most elements in a tile
    std::vector<int> nptr;             // per tile: first active node (ntiles + 1)
    std::vector<int> eptr, elist;      // per tile: its elements (internal ids)
    std::vector<unsigned char> tj;     // per gather term: index of its element in the tile's list
};

// Fails (false, with why) only when one node alone reads more than
// emax_limit elements.
bool build_mma_tiles(const Plan &P, int tn, int emax_limit, MmaTiles &T, std::string &why);

// Per active node, the FP32 step's node coefficients: 1/m_full (x, y) and
// -2 a2 C (x, y).
pvec<float> node_coef32(const Plan &P);

// Fixed-size gather records of the FP32 direct gather: per active node its
// first four element terms (tlist entries, in tlist order; -1 past the last)
// and 1/m_full, so that a common node reads no list pointers, no node
// coefficients and no DRM or anchor lists, and its term entries are one
// 16-byte load with nothing before it in the gather chain.  A node with more
// than four terms, DRM terms, anchored hanging nodes, a dashpot or unequal x
// and y coefficients is marked by a negative invm and reads those parts from
// the CSR lists and node coefficients (its terms past the fourth from
// tlist[tptr[n] + 4 ...]).  nc is node_coef32(P).  Fails (false, with why)
// when an entry would not fit 31 bits (2^28 elements or more).
struct NodeSlots {
    pvec<int> slot4;                   // 4 per active node
    pvec<float> invm;                  // per active node: 1/m_full (x = y), or -1 on a marked node
    long long marked = 0;              // marked nodes
};
bool build_node_slots(const Plan &P, const pvec<float> &nc, NodeSlots &out, std::string &why);

// What the bulk-copy pipeline reads per tile, in the formats its kernel
// decodes (all arrays of 32-bit words, every tile's part 16-byte aligned):
//   hdr    4 per tile: halo nodes, terms, term-pack offset (16-byte units), runs
//   runs   2 * max_runs per tile: (first node, count), count 0 past the last
//   nrec   8 per active node: 1/m_full x, y and -2 a2 C x, y (float bits);
//          first term in the tile | terms << 16; halo slot of the node;
//          DRM start | count << 24; anchor-link start | count << 24
//   tpack  per tile: the halo slots of each term's element corners as
//          ushort4 (the node's corner in bits 14-15 of the first slot), an
//          even number of them, then each term's (A, B, C, D) times its
//          weight (1 or 1/2) as float bits
// Returns false (with why) when the model exceeds a field of these formats.
struct PipePack {
    std::vector<int> hdr, runs, nrec, tpack;
    int tmax = 0;                      // most terms in a tile
};
bool build_pipe_pack(const Plan &P, const Tiles &T, int max_runs, PipePack &out, std::string &why);

// Build the plan.  Returns EXFEM_OK or an EXFEM_E_* code with err filled.
// r_internal > prob.nrhs pads the right-hand sides with zero-amplitude waves
// (see padded_rhs); the plan's arrays then carry r_internal of them.
// fp64_operator false (an FP32 context) leaves out the arrays only the FP64
// kernels read: the per-element calck values, FP64 closed-form coefficients
// and (mu, lambda) pairs (ekv, ecoef, emulam stay empty).
int build_plan(const exfem_mesh &mesh, const exfem_problem &prob, bool reorder, Plan &plan, std::string &err,
               int r_internal = 0, bool fp64_operator = true);

// Internal right-hand-side count of the FP32 form for R of the caller's.  A
// node's row holds R floats; when R is odd its rows are not 8-byte aligned,
// straddle L1 sectors and run one value per thread, and the few-RHS step is
// L1-bound.  Zero-amplitude padding to an even count, and to a multiple of 4
// from 14 (four per thread), measured 10-18% faster per step on 1.4e5-6e5
// element valleys with R = 9, 13 and 15, the padding's work included.
inline int padded_rhs(int R) {
    if (R <= 2) return R;
    int p = R + (R & 1);
    if (p >= 14 && (p & 3) != 0) p += 2;
    return p;
}

}  // namespace exfem
