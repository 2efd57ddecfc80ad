// host_system.hpp - host-side mirror of the reference's system assembly:
// Topology, extract_interaction_group, the force-field generators of the
// hot path and SystemGenerator, plus the compile step that lays a generated
// system out for the kernels.
#pragma once
#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <map>
#include <memory>
#include <optional>
#include <set>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "engine_types.h"

namespace ocm {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// ---------------------------------------------------------------------------
// Tables (src/util/Constants.hpp:26-102).
// ---------------------------------------------------------------------------
constexpr double kFlaThetaMin = 1.30900;
constexpr double kFlaThetaMax = 2.87979;
const std::array<double, 10>* fla_spline_table(const std::string& aa);
const std::array<double, 10>* fla_second_derivative_table(const std::string& aa);
const std::array<double, 7>* fld_fourier_table(const std::string& key);
const std::vector<std::string>& fld_table_keys();  // std::map order of the reference
const std::vector<std::string>& amino_acids();     // 20 codes, std::map order

// Physical constants used by the generators (Constants.hpp:16-23 and the
// OpenMM unit constants they rely on).
namespace constant {
constexpr double Na = 6.02214076e23;
constexpr double kB = 1.380649e-23;
constexpr double pi = 3.1415926535897932385;
constexpr double elementary_charge = 1.6021766208e-19;
constexpr double eps0 = 8.854187817e-12 * 1.0e3 * 1.0e-9 / Na;  // C^2 mol/kJ/nm
constexpr double boltz = 0.00831446261815324;                   // kJ/mol/K (NA*kB/1000)
}  // namespace constant

// ---------------------------------------------------------------------------
// Topology (src/Topology.hpp / Topology.cpp).
// ---------------------------------------------------------------------------
class Topology {
  public:
    explicit Topology(std::size_t n) : nodes_(n) {}
    void add_edges(const std::vector<std::pair<std::size_t, std::size_t>>& edges,
                   const std::string& type);
    void make_molecule(const std::string& type);
    std::vector<std::pair<std::size_t, std::size_t>> ignore_list_within_molecule() const;
    std::vector<std::pair<std::size_t, std::size_t>> ignore_list_within_edge(
        std::size_t dist, const std::string& type) const;
    std::size_t size() const { return nodes_.size(); }

  private:
    int type_id(const std::string& type);
    int find_type(const std::string& type) const;
    void collect_within(std::size_t node, std::size_t dist, int type,
                        std::vector<std::size_t>& out) const;
    std::vector<std::vector<std::pair<std::size_t, int>>> nodes_;
    std::vector<std::string> types_;
    std::vector<std::vector<std::size_t>> molecules_;
    bool molecule_updated_ = false;
};

using IndexPairs = std::vector<std::pair<int64_t, int64_t>>;
using GroupPairs = std::vector<std::pair<std::set<int>, std::set<int>>>;

// extract_interaction_group (InteractionGroup.hpp:17-101) over "has value"
// flags and integer group ids (-1 = no group).
GroupPairs extract_interaction_group(const std::vector<bool>& has_value,
                                     const std::vector<std::pair<int, int>>& ignore_group_pairs,
                                     const std::vector<int>& group_vec);

// ---------------------------------------------------------------------------
// Generated forces: what a generator's generate() hands to the System.
// ---------------------------------------------------------------------------
enum class ForceKind { HarmonicBond, GoContact, FlexibleLocalAngle, FlexibleLocalDihedral,
                       ExcludedVolume, DebyeHuckel, LennardJonesRepulsive,
                       LennardJonesAttractive, GaussianBond, GaussianDihedral,
                       WeeksChandlerAndersen, CappedGoContact };

struct GeneratedForce {
    ForceKind kind;
    std::string name;
    int group = 0;
    bool periodic = false;
    // explicit terms
    std::vector<std::array<int64_t, 4>> idx;
    std::vector<std::array<double, 3>> par;
    // FlexibleLocalAngle
    std::array<double, 10> spline_y{};
    double theta_min = 0, theta_max = 0, min_energy = 0;
    // FlexibleLocalDihedral
    std::array<double, 7> fourier{};
    // pair terms
    double cutoff = 0, switch_distance = -1;
    double eps = 0, cutoff_correction = 0, k_e = 0, debye_length = 0;
    std::vector<double> pp0, pp1;  // per-particle parameters (NaN = none)
    IndexPairs exclusions;
    GroupPairs groups;
};

class ForceFieldGeneratorBase {
  public:
    virtual ~ForceFieldGeneratorBase() = default;
    virtual GeneratedForce generate() const = 0;
    virtual std::string name() const = 0;
};

class HarmonicBondForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    HarmonicBondForceFieldGenerator(std::vector<std::pair<int64_t, int64_t>> idx,
                                    std::vector<double> v0s, std::vector<double> ks,
                                    bool use_periodic);
    GeneratedForce generate() const override;
    std::string name() const override { return "HarmonicBond"; }
  private:
    std::vector<std::pair<int64_t, int64_t>> idx_;
    std::vector<double> v0s_, ks_;
    bool periodic_;
};

class GoContactForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    GoContactForceFieldGenerator(std::vector<std::pair<int64_t, int64_t>> idx,
                                 std::vector<double> ks, std::vector<double> r0s,
                                 bool use_periodic);
    GeneratedForce generate() const override;
    std::string name() const override { return "GoContact"; }
  private:
    std::vector<std::pair<int64_t, int64_t>> idx_;
    std::vector<double> ks_, r0s_;
    bool periodic_;
};

// GaussianBondForceFieldGenerator (GaussianBondForceFieldGenerator.hpp:22-48,
// .cpp:3-23): k exp(-(r - v0)^2 / (2 sigma^2)).
class GaussianBondForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    GaussianBondForceFieldGenerator(std::vector<std::pair<int64_t, int64_t>> idx,
                                    std::vector<double> ks, std::vector<double> v0s,
                                    std::vector<double> sigmas, bool use_periodic);
    GeneratedForce generate() const override;
    std::string name() const override { return "GaussianBond"; }
  private:
    std::vector<std::pair<int64_t, int64_t>> idx_;
    std::vector<double> ks_, v0s_, sigmas_;
    bool periodic_;
};

// GaussianDihedralForceFieldGenerator (GaussianDihedralForceFieldGenerator.hpp,
// .cpp:3-27): k exp(-dphi^2 / (2 sigma^2)) with dphi wrapped to [-pi, pi).
class GaussianDihedralForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    GaussianDihedralForceFieldGenerator(std::vector<std::array<int64_t, 4>> idx,
                                        std::vector<double> ks, std::vector<double> theta0s,
                                        std::vector<double> sigmas, bool use_periodic);
    GeneratedForce generate() const override;
    std::string name() const override { return "GaussianDihedral"; }
  private:
    std::vector<std::array<int64_t, 4>> idx_;
    std::vector<double> ks_, theta0s_, sigmas_;
    bool periodic_;
};

class FlexibleLocalAngleForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    FlexibleLocalAngleForceFieldGenerator(std::vector<std::array<int64_t, 3>> idx,
                                          std::vector<double> ks,
                                          const std::array<double, 10>& spline_table,
                                          const std::string& aa_name, bool use_periodic,
                                          double min_theta = kFlaThetaMin,
                                          double max_theta = kFlaThetaMax);
    GeneratedForce generate() const override;
    std::string name() const override { return "FlexibleLocalAngle (" + aa_ + ")"; }
    double spline_interpolate(double th) const;
  private:
    std::vector<std::array<int64_t, 3>> idx_;
    std::vector<double> ks_;
    std::string aa_;
    double min_theta_, max_theta_, dtheta_, rdtheta_;
    std::array<double, 10> y_, d2y_, thetas_;
    bool periodic_;
};

class FlexibleLocalDihedralForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    FlexibleLocalDihedralForceFieldGenerator(std::vector<std::array<int64_t, 4>> idx,
                                             std::vector<double> ks,
                                             const std::array<double, 7>& fourier_table,
                                             const std::string& aa_pair_name,
                                             bool use_periodic);
    GeneratedForce generate() const override;
    std::string name() const override { return "FlexibleLocalDihedral (" + pair_ + ")"; }
  private:
    std::vector<std::array<int64_t, 4>> idx_;
    std::vector<double> ks_;
    std::array<double, 7> f_;
    std::string pair_;
    bool periodic_;
};

struct PairGeneratorCommon {
    IndexPairs ignore_list;
    bool use_periodic = false;
    std::vector<std::pair<int, int>> ignore_group_pairs;
    std::vector<int> group_vec;
};

class ExcludedVolumeForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    ExcludedVolumeForceFieldGenerator(double eps, double cutoff, std::vector<double> radii,
                                      PairGeneratorCommon common);
    GeneratedForce generate() const override;
    std::string name() const override { return "ExcludedVolume"; }
  private:
    double eps_, cutoff_;
    std::vector<double> radii_;
    PairGeneratorCommon c_;
    GroupPairs groups_;
};

class DebyeHuckelForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    DebyeHuckelForceFieldGenerator(double ionic_strength, double temperature,
                                   double cutoff_ratio, std::vector<double> charges,
                                   PairGeneratorCommon common);
    GeneratedForce generate() const override;
    std::string name() const override { return "DebyeHuckel"; }
    static double dielectric_water(double T, double C);
  private:
    double ratio_;
    std::vector<double> q_;
    PairGeneratorCommon c_;
    GroupPairs groups_;
    double debye_length_, inv_4_pi_eps0_epsk_, cutoff_correction_, abs_cutoff_;
};

class LennardJonesForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    LennardJonesForceFieldGenerator(bool attractive, double cutoff_ratio,
                                    std::vector<double> eps, std::vector<double> sigma,
                                    PairGeneratorCommon common);
    GeneratedForce generate() const override;
    std::string name() const override {
        return attractive_ ? "LennardJonesAttractive" : "LennardJonesRepulsive";
    }
  private:
    bool attractive_;
    double ratio_;
    std::vector<double> eps_, sigma_;
    PairGeneratorCommon c_;
    GroupPairs groups_;
};

// WeeksChandlerAndersenForceFieldGenerator (WeeksChandlerAndersenForceFieldGenerator.cpp:9-113):
// step(2^(1/6) s - r) (4 e ((s/r)^12 - (s/r)^6) + e) with s the arithmetic and
// e the geometric mean of the pair's parameters; cutoff 2^(1/6) (s_max + s_2nd) / 2.
class WeeksChandlerAndersenForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    WeeksChandlerAndersenForceFieldGenerator(std::vector<double> sigmas, std::vector<double> eps,
                                             PairGeneratorCommon common);
    GeneratedForce generate() const override;
    std::string name() const override { return "WeeksChandlerAndersen"; }
  private:
    std::vector<double> sigma_, eps_;
    PairGeneratorCommon c_;
    GroupPairs groups_;
};

// Uniform pair generators: one sigma and epsilon for every pair between the
// particle sets `former` and `latter`.
//  * UniformWeeksChandlerAndersenForceFieldGenerator (UniformWeeksChandlerAndersenForceFieldGenerator.cpp:9-185):
//    4 e ((s/r)^12 - (s/r)^6 + 1/4), cutoff 2^(1/6) s;
//  * UniformLennardJonesAttractiveForceFieldGenerator (UniformLennardJonesAttractiveForceFieldGenerator.cpp:11-189):
//    e (step(r - t) 4 ((s/r)^12 - (s/r)^6) - step(t - r)), t = 2^(1/6) s,
//    cutoff s * cutoff_ratio, switched from 0.9 cutoff.
class UniformPairForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    UniformPairForceFieldGenerator(bool attractive, int64_t system_size, double eps, double sigma,
                                   double cutoff_ratio, std::vector<int64_t> former,
                                   std::vector<int64_t> latter, PairGeneratorCommon common);
    GeneratedForce generate() const override;
    // the reference's own spelling of the WCA name
    std::string name() const override {
        return attractive_ ? "UniformLennardJonesAttractive" : "UniformWeeksChadlerAndersen";
    }
  private:
    bool attractive_;
    int64_t n_;
    double eps_, sigma_, ratio_;
    PairGeneratorCommon c_;
    GroupPairs groups_;
};

// CappedGoContactForceFieldGenerator (CappedGoContactForceFieldGenerator.hpp:14-47,
// .cpp:5-31): the Go 10-12 form beyond cap * r0, its linear continuation
// k (slope r / r0 + intercept) below.
class CappedGoContactForceFieldGenerator final : public ForceFieldGeneratorBase {
  public:
    CappedGoContactForceFieldGenerator(std::vector<std::pair<int64_t, int64_t>> idx,
                                       std::vector<double> ks, std::vector<double> r0s,
                                       double capping_ratio, bool use_periodic);
    GeneratedForce generate() const override;
    std::string name() const override { return "CappedGoContact"; }
  private:
    std::vector<std::pair<int64_t, int64_t>> idx_;
    std::vector<double> ks_, r0s_;
    double cap_;
    bool periodic_;
};

// ---------------------------------------------------------------------------
// SystemGenerator (src/SystemGenerator.cpp:4-111).
// ---------------------------------------------------------------------------
struct SystemDesc {
    std::vector<double> masses;
    bool periodic_box = false;
    double box[3] = {0, 0, 0};
    std::vector<GeneratedForce> forces;
    std::vector<std::string> group_names;  // index = group id
};

class SystemGenerator {
  public:
    explicit SystemGenerator(std::vector<double> masses) { desc_.masses = std::move(masses); }
    void set_pbc(double x, double y, double z);
    // Returns the force group the generator's force lands in.
    int add_ff_generator(std::unique_ptr<ForceFieldGeneratorBase> gen);
    const SystemDesc& desc() const { return desc_; }
    std::string describe_json() const;
  private:
    SystemDesc desc_;
    std::map<std::string, int> group_of_name_;
};

// ---------------------------------------------------------------------------
// Compiled layout consumed by the engines.
// ---------------------------------------------------------------------------
struct CompiledSystem {
    int64_t n = 0;
    bool periodic = false;      // pair terms use the minimum image
    double box[3] = {0, 0, 0};
    std::vector<float> inv_mass;
    std::vector<float> p0, p1;  // float4 per particle (4*n each)
    std::vector<uint32_t> labels;
    PairConsts pc{};
    int slot_group[kNumSlots];  // force group of each energy slot, -1 = absent
    std::vector<BondTerm> bonds;
    std::vector<AngleTerm> angles;
    std::vector<DihedralTerm> dihedrals;
    std::vector<FlaTable> fla;
    std::vector<FldTable> fld;
    // exclusions: CSR over particles (both directions), bits = kTerm* excluded
    std::vector<int32_t> ex_start, ex_j;
    std::vector<uint8_t> ex_bits;
    double max_cutoff = 0;
    bool lj_same_sigma = false;  // both LJ terms present with equal per-particle sigma
};

CompiledSystem compile_system(const SystemDesc& d);

// Natural cubic spline second derivatives (zero at both ends) through
// equidistant nodes (OpenMM Continuous1DFunction, non-periodic).
std::array<double, 10> natural_spline_second_derivatives(const std::array<double, 10>& y,
                                                         double h);

}  // namespace ocm
