// engine_types.h - plain-old-data layouts shared by host code and kernels.
#pragma once
#include <cstdint>

namespace ocm {

// Fixed point: 2^32 units per kJ/mol/nm (int64 accumulators).
constexpr float kFixedScaleF = 4294967296.0f;
constexpr double kFixedInv = 1.0 / 4294967296.0;
constexpr float kTwoPow1_3 = 1.2599210498948732f;  // (2^(1/6))^2

// Pair-term bits (also the order of per-term 4-bit labels and mask words).
constexpr int kTermEXV = 1;
constexpr int kTermDH = 2;
constexpr int kTermLJR = 4;
constexpr int kTermLJA = 8;
constexpr int kNumPairTerms = 4;
// Kernel-template flag (not a term): the attractive LJ term's sigma equals
// the repulsive one's for every particle, so sigma mixing and the s^6, s^12
// powers are formed once per pair.  The results are bit-identical.
constexpr int kLJSameSigma = 16;

// Energy slots (one per term kind); mapped to force groups on the host.
enum EnergySlot {
    kSlotEXV = 0,
    kSlotDH = 1,
    kSlotLJR = 2,
    kSlotLJA = 3,
    kSlotHB = 4,
    kSlotGO = 5,
    kSlotFLA = 6,
    kSlotFLD = 7,
    kSlotGB = 8,   // Gaussian bond (AICG2+)
    kSlotGD = 9,   // Gaussian dihedral (AICG2+)
    kSlotCGO = 10, // capped Go contact
    kNumSlots = 11
};

constexpr int kBondHarmonic = 0;
constexpr int kBondGo = 1;
constexpr int kBondGauss = 2;
constexpr int kBondCappedGo = 3;

// Energy slot of a bond kind.
#if defined(__CUDACC__)
__host__ __device__
#endif
inline int bond_slot(int kind) {
    return kind == kBondHarmonic ? kSlotHB : kind == kBondGo ? kSlotGO : kind == kBondGauss ? kSlotGB : kSlotCGO;
}

constexpr int kDihFLD = 0;
constexpr int kDihGauss = 1;

// Philox4x32-10 constants (Salmon et al. 2011).
constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;
constexpr uint32_t kPhiloxKey1 = 0x6F636D31u;  // second key word, xor-ed with the stream id
constexpr uint32_t kPurposeLangevin = 0u;
constexpr uint32_t kPurposeVelocityInit = 1u;

// Constants of the fused pair kernel for one system.
struct PairConsts {
    float exv_eps, exv_rc2, exv_inv_rc2;
    float dh_k, dh_inv_lambda, dh_inv_lambda_log2e, dh_rc2, dh_corr;
    float ljr_rc2;
    float lja_rc2, lja_rs, lja_inv_width;
    float list_rc2;  // largest pair cutoff squared
    int terms;       // kTerm* bits present
    int uses_labels; // bit t: term t has interaction groups
    int ljr_geometric;  // repulsive LJ slot mixes epsilon geometrically (WCA): p0.z holds sqrt(eps)
    unsigned long long allow[kNumPairTerms];  // label-pair matrix per term (8x8 bits)
};

// Natural cubic spline table of one FlexibleLocalAngle force.
struct FlaTable {
    float theta_min, theta_max, inv_h, emin;
    float y[10];
    float m[10];  // second derivatives * h^2 / 6
};

// Fourier table of one FlexibleLocalDihedral force.
struct FldTable {
    float c[7];   // c, kcos1, ksin1, kcos2, ksin2, kcos3, ksin3
    float emin;
};

// Explicit bond-like term (harmonic bond, Go contact or Gaussian bond).
struct BondTerm {
    int32_t i, j;
    int32_t kind;      // kBondHarmonic / kBondGo / kBondGauss / kBondCappedGo
    int32_t periodic;  // minimum image when nonzero
    float p0, p1;      // (r0, k) harmonic; (k, r0) Go; (k, 1 / (2 sigma^2)) Gaussian; (k, 1 / cap) capped Go
    float r0sq_hi, r0sq_lo;  // r0^2 (v0^2 for the Gaussian) as an unevaluated float sum
};
struct AngleTerm {
    int32_t i, j, k, table;
    float kk;
    int32_t periodic;
};
struct DihedralTerm {
    int32_t i, j, k, l;
    int32_t table, periodic;  // table: FLD Fourier table (kDihFLD)
    float kk;
    int32_t kind;             // kDihFLD / kDihGauss
    float theta0, inv2s2;     // Gaussian: centre (rad) and 1 / (2 sigma^2)
};

// Langevin constants of one system (OpenMM LangevinIntegrator).
struct LangevinConsts {
    float vscale;    // exp(-gamma dt)
    float fscale;    // (1 - vscale)/gamma, or dt when gamma == 0
    float noise;     // sqrt(kT (1 - vscale^2))
    float dt;
    uint32_t seed;
    uint32_t stream;
};

}  // namespace ocm
