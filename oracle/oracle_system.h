// oracle_system.h - TEST INFRASTRUCTURE, not part of the engine.
//
// The flat system description shared by the FP64 oracle (ocm_oracle.cpp)
// and the timed FP32 CPU restatement (cpu_baseline.cpp), plus the oracle
// helpers the restatement reuses for its set-up.
#pragma once
#include <cstdint>

extern "C" {

// Flat description of one system in the units the generators receive.
typedef struct OracleSystem {
    int64_t n;
    const double* pos;  // 3n
    int periodic;
    double box[3];
    // harmonic bonds: k is the OpenMM 1/2 k (r - r0)^2 constant
    int64_t n_bonds;
    const int64_t* bond_idx;
    const double* bond_v0;
    const double* bond_k;
    int bond_periodic;
    // Go contacts
    int64_t n_go;
    const int64_t* go_idx;
    const double* go_k;
    const double* go_r0;
    int go_periodic;
    // flexible-local angles: centre-residue table index (0..19)
    int64_t n_fla;
    const int64_t* fla_idx;
    const double* fla_k;
    const int32_t* fla_aa;
    // flexible-local dihedrals: the two residue indices of the "AAA-BBB" coef
    int64_t n_fld;
    const int64_t* fld_idx;
    const double* fld_k;
    const int32_t* fld_aa1;
    const int32_t* fld_aa2;
    // pair terms; *_ign_bond / *_ign_contact: exclusion distance along
    // "bond" / "contact" edges (-1: none)
    int exv_on;
    double exv_eps, exv_ratio;
    const double* exv_radius;
    int exv_ign_bond, exv_ign_contact;
    int dh_on;
    double dh_I, dh_T, dh_ratio;
    const double* dh_q;
    int dh_ign_bond, dh_ign_contact;
    int ljr_on;
    double ljr_ratio;
    const double* ljr_eps;
    const double* ljr_sigma;
    int ljr_ign_bond, ljr_ign_contact;
    int lja_on;
    double lja_ratio;
    const double* lja_eps;
    const double* lja_sigma;
    int lja_ign_bond, lja_ign_contact;
    int fp32_cutoff;  // decide r < rc on the engine's FP32 r^2
    // pair enumeration: 0 all pairs, 1 cell grid, -1 cell grid above 4096 beads
    int pair_cells;
    // AICG2+ Gaussian bonds k exp(-(r - v0)^2 / (2 sigma^2)) and dihedrals
    // k exp(-dphi^2 / (2 sigma^2)) (theta0, sigma in radians)
    int64_t n_gb;
    const int64_t* gb_idx;
    const double* gb_k;
    const double* gb_v0;
    const double* gb_sigma;
    int gb_periodic;
    int64_t n_gd;
    const int64_t* gd_idx;
    const double* gd_k;
    const double* gd_theta0;
    const double* gd_sigma;
    int gd_periodic;
    // WeeksChandlerAndersen in the repulsive LJ slot: geometric epsilon mean
    // (WeeksChandlerAndersenForceFieldGenerator.cpp:38-45)
    int ljr_geometric;
    // uniform generators: per-particle side bits (1 former, 2 latter); a
    // pair interacts if one is former and the other latter; null = all
    const int8_t* ljr_side;
    const int8_t* lja_side;
    // capped Go contacts (CappedGoContactForceFieldGenerator.cpp:5-31)
    int64_t n_cgo;
    const int64_t* cgo_idx;
    const double* cgo_k;
    const double* cgo_r0;
    const double* cgo_cap;   // capping ratio per contact
    int cgo_periodic;
    int cgo_contact_edges;   // the contacts are "contact" edges of the topology
    // group-based ignores (InteractionGroup.hpp:19-99): per-particle group
    // id (-1 none) and, per pair term (EXV, DH, LJR, LJA), the ignored
    // (group, group) pairs, symmetric
    const int32_t* grp;
    int64_t n_igp[4];
    const int32_t* igp[4];
    // molecule-based ignores per pair term: no pair inside one molecule (the
    // connected components of the bond edges, Topology.cpp:7-73)
    int ign_molecule[4];
} OracleSystem;

// Helpers exported by ocm_oracle.cpp.
int oracle_dh_params(double I, double T, double ratio, double* out5);
double oracle_fla_min_energy(int aa);
double oracle_fld_min_energy(int cls);
int oracle_natural_spline(const double* y10, double h, double* M10);
int oracle_fld_classes(int aa1, int aa2, int32_t* out, int cap);
int oracle_ignore_within(int64_t n, int64_t n_bond, const int64_t* bonds, int64_t n_contact,
                         const int64_t* contacts, int ign_bond, int ign_contact, int64_t* out,
                         int64_t cap, int64_t* n_out);
void oracle_top_two(const double* v, int64_t n, int strict, double* out2);

}  // extern "C"
