// Device plan of the sparse HEOM Liouvillian: the reference's per-ADO COO data and
// coupling tables recompiled into flat gather lists for one-thread-per-entry kernels.
#pragma once
#include <cstdint>
#include <vector>

#include "common.h"

namespace heom {

// Coupling coefficient encoding (CoupRec.cid): bit 31 = take conj of the source value;
// bit 30 = unit pair cL = i*sL, cR = i*sR with sL = -1 if bit 0, sR = -1 if bit 1
// (the higher-tier and RDO couplings, which need no multiplication); otherwise
// bits 0..29 index the coefficient tables (the lower-tier cb/cd pairs).
constexpr int32_t kCoefConj = (int32_t)0x80000000;
constexpr int32_t kCoefUnit = 0x40000000;

// Packed coupling record: source segment offset, map base, coefficient id and conj bit.
struct CoupRec {
    int32_t src_off;   // entry offset of the source ADO in the vector
    int32_t map_base;  // offset of this coupling's gather map (one word per output entry)
    int32_t cid;       // coefficient pair id; bit 31 = take conj of the source value
    int32_t pad;
};

// Structure of one plan (forward or adjoint).  All indices are 0-based.
struct HostPlan {
    int64_t lunk = 0;                       // entries; the trace slot is entry lunk
    int32_t nado = 0;                       // ADOs with at least one stored entry
    int32_t nslots = 0;                     // nalf * nspin lead-shift slots (<= 4)
    int32_t nh = 0;                         // entries of the Hamiltonian structure
    std::vector<int32_t> ent_ado;           // lunk
    std::vector<int32_t> ado_off;           // nado + 1
    std::vector<int32_t> ado_cls;           // nado
    std::vector<int32_t> ado_cnt;           // nado: 4 signed int8 counts of sum(dipm) per slot
    std::vector<cd> g0;                     // nado: sum of cgamma over the drawers
    std::vector<int32_t> coup_ptr;          // nado + 1
    std::vector<int32_t> coup_mid;          // nado: first unit-coefficient coupling of the ADO
                                            // (its couplings are ordered coefficient pairs first)
    std::vector<CoupRec> coup;
    std::vector<uint32_t> maps;             // word: lo16 = left src (q+1, bit15 = minus), hi16 = right
    std::vector<cd> cl, cr;                 // coefficient pairs
    std::vector<int8_t> coef_kind;          // 1 = lower-tier (cb/cd) pair, 0 = otherwise
    std::vector<int32_t> cls_tptr;          // per class: base of its row pointers in term_ptr
    std::vector<int32_t> term_ptr;          // concatenated CSR row pointers of same-tier terms
    std::vector<uint32_t> terms;            // q | hidx << 16 | side << 31 (side 1 = right, i*x*H)
    std::vector<int32_t> trace_idx;         // forward plan: RDO diagonal entries summed into the trace slot
    int32_t adjoint = 0;
    // bookkeeping for measurement
    int64_t n_terms_same = 0, n_couplings = 0, n_maps = 0, n_classes = 0;
    double gather_hits = 0;                 // nonzero map words (useful gathers) per apply
};

// H structure shared by both plans: the (row, col) pairs whose values drive the
// same-tier commutator; values are given per parameter set.
struct HStructure {
    int n = 0;
    std::vector<int32_t> idx;               // dense n*n -> structure index or -1
    std::vector<int32_t> rows, cols;        // structure entries
};

HStructure make_hstructure(const heom_tables &t, const std::vector<const double _Complex *> &extra);
void build_forward_plan(const heom_tables &t, const HStructure &hst, HostPlan &out);
void build_adjoint_plan(const heom_tables &t, const HostPlan &fwd, HostPlan &out);
// Order every ADO's couplings as coefficient pairs first, then unit pairs (stable, so each
// kind keeps its order), and record the boundary in coup_mid.
void split_couplings(HostPlan &P);
// Plan of the correlation-function operator on the pattern cf: entries [h; a], no trace slot
// (corrfunc/calc_ax_cf_spa_omp.f90)
void build_cf_plan(const heom_tables &t, const heom_cf_tables &cf, const HStructure &hst, HostPlan &out);
// plan bytes one apply reads: coupling records (16 B), one map word per record and output
// entry (4 B), the per-entry ADO index (4 B) and the per-ADO arrays (g0 16 B + 4 ints)
double plan_read_bytes(const HostPlan &P);
// derivative coefficient table of the forward plan w.r.t. a common linewidth scale:
// lower-tier pairs divided by gamma, everything else zero
void gamma_derivative_coefs(const heom_tables &t, const HostPlan &fwd, double gamma, std::vector<cd> &cl, std::vector<cd> &cr);

}  // namespace heom
