// engine.hpp - host classes of the plain (single-system) and batched engines.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "host_system.hpp"

namespace ocm {

void cuda_check(cudaError_t e, const char* what);
#define OCM_CK(x) ::ocm::cuda_check((x), #x)

// Owning device buffer.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            throw Error(3, std::string("[error] device allocation of ") +
                               std::to_string(count * sizeof(T)) + " bytes failed: " +
                               cudaGetErrorString(e));
        }
        n = count;
    }
    void upload(const std::vector<T>& v, cudaStream_t s) {
        if (v.size() > n) alloc(v.size());
        if (!v.empty())
            OCM_CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    }
};

// Periodic box in FP64 (L, 1/L per axis) as the kernels take it.
struct BoxD {
    double L[3], iL[3];
    int periodic;
};

struct ListFlags {
    // kBlownUp: a force contribution or a summed force of 1e9 kJ/mol/nm or
    // more (the fixed-point accumulators hold about 2.1e9), a non-finite
    // force, velocity or position
    enum : int { kTileOverflow = 1, kMaskOverflow = 2, kSkinViolation = 4, kChargedOverflow = 8, kBlownUp = 16 };
};

class BatchEngine;

// Device-resident single system, the part of an OpenMM Context + Langevin
// integrator that the reference drives through Simulator::run.
class PlainContext {
  public:
    PlainContext(const SystemDesc& d, double temperature, double friction, double dt,
                 int32_t seed, int device);
    ~PlainContext();
    void set_positions(const double* xyz);
    void get_positions(double* xyz);
    void set_velocities(const double* v);
    void get_velocities(double* v);
    void set_velocities_to_temperature(double temperature, int32_t seed);
    void get_state(uint32_t groups, double* forces, double* energy);
    void group_energies(double* energies32);
    double kinetic_energy();
    void step(int64_t n);
    // Engine of step(): kEngineAuto runs a non-periodic system of at most
    // kOneSystemMaxBeads beads as a one-system persistent launch of the
    // batched kernel (one SM: no per-step launches, no grid-wide list
    // build) and every other system on the cluster-pair tiles;
    // kEngineTiles / kEngineOneSystem force one or the other.
    enum { kEngineAuto = 0, kEngineTiles = 1, kEngineOneSystem = 2 };
    static constexpr int64_t kOneSystemMaxBeads = 512;
    void set_engine(int32_t mode);
    bool last_step_one_system() const { return last_step_one_system_; }
    void set_list_options(int32_t interval, double skin);
    void list_pairs(int64_t* out, int64_t cap, int64_t* n_out);
    void cluster_order(int64_t* out, int64_t cap, int64_t* n_out);
    // L-BFGS local energy minimisation (minimize.cpp); returns the iterations
    int64_t minimize(double tolerance, int64_t max_iterations);
    // Why the last minimisation stopped (kMin*) and its final RMS force.
    enum { kMinConverged = 0, kMinIterationCap = 1, kMinStagnated = 2, kMinLineSearch = 3 };
    int32_t min_reason = -1;
    double min_rms = 0.0;
    bool charged_split() const { return charged_split_; }
    double tile_cutoff() const { return tile_cutoff_; }
    int64_t charged_pairs() const { return charged_last_; }

    int device = 0;
    int64_t n = 0, np = 0, nc = 0;
    int64_t steps_done = 0, list_builds = 0;
    int32_t rebuild_interval = 10;
    double skin = 0.25;
    bool reorder = false;
    int64_t tiles_last = 0, masked_last = 0;
    CompiledSystem cs;

  private:
    void rebuild(cudaStream_t s);
    void launch_forces(cudaStream_t s, bool energy, uint32_t slots_enabled, int r);
    void launch_integrate(cudaStream_t s, int r);
    void ensure_capacity();
    cudaGraphExec_t graph_for(int chunk);
    void clear_graphs();
    void setup_charged_cells();
    void setup_columns(double width);
    BoxD box_d() const;
    float wrap_pad() const;
    void alloc_tile_arrays();
    bool eval(uint32_t groups, bool energy, double* forces, double* slot_energy);
    uint32_t slots_for_groups(uint32_t groups) const;
    void check_positions_set() const;
    // positions from the minimiser: no re-estimate of the cluster column width
    void set_positions_internal(const double* xyz);
    void set_positions_impl(const double* xyz, bool retune);

    bool one_system_eligible();
    void step_one_system(int64_t nsteps);

    SystemDesc desc_;  // kept for the one-system batch
    int32_t engine_mode_ = kEngineAuto;
    std::unique_ptr<BatchEngine> one_;
    int64_t one_slot_ = -1;
    bool one_refused_ = false;  // the batched kernel does not take this system
    bool last_step_one_system_ = false;
    int32_t one_seed_ = 0;
    double one_T_ = 0, one_friction_ = 0, one_dt_ = 0;
    cudaStream_t stream_ = nullptr;
    std::map<int, cudaGraphExec_t> graphs_;
    bool positions_set_ = false;
    LangevinConsts lc_{};
    int cell_dims_[3] = {1, 1, 1};
    int num_sms_ = 1;
    int64_t n_cells_ = 0;
    int64_t tile_cap_ = 0, mask_cap_ = 0;
    float3 box_{0, 0, 0}, inv_box_{0, 0, 0};
    // Charged-pair list: when the Debye-Hueckel cutoff is the largest, the
    // tiles serve the other pair terms only and every charged bead gets a
    // row of its charged partners within the Debye-Hueckel cutoff (+ skin),
    // built from a cell grid over the charged beads.
    bool charged_split_ = false;
    double tile_cutoff_ = 0;  // largest cutoff the tiles serve
    int charged_cells_[3] = {1, 1, 1};
    int64_t n_charged_ = 0, n_charged_cells_ = 0, charged_last_ = 0;
    int64_t chg_row_cap_ = 0;  // entries per charged bead's row

    // per particle (original order)
    DevBuf<double> x_, y_, z_;
    DevBuf<float> vx_, vy_, vz_, invm_;
    DevBuf<unsigned long long> F_;  // 3*n, SoA
    DevBuf<float4> xq_, xlo_, ref_, p0_, p1_;  // xlo: FP64 remainder of the FP32 position
    DevBuf<uint32_t> lab_;
    DevBuf<int32_t> slot_;
    // cluster order
    DevBuf<int32_t> perm_;
    DevBuf<float4> xs_, p0s_, p1s_;
    DevBuf<uint32_t> labs_;
    DevBuf<float4> bb_c_, bb_h_;
    DevBuf<float4> anc_, ext_;  // cluster anchors, largest anchored offset per axis
    DevBuf<int32_t> tile_count_, tile_start_, tile_j_, tile_mask_;
    DevBuf<float4> tile_shift_;  // per tile: anchor shift, w != 0 when the minimum image is needed
    DevBuf<int32_t> tile_i_;     // per tile: its row cluster
    DevBuf<int32_t> raw_start_, raw_i_, raw_j_;  // candidate tiles before pruning
    DevBuf<uint8_t> keep_;
    DevBuf<uint32_t> masks_;
    DevBuf<int32_t> mask_count_;
    // cluster order: columns in x-y, each sorted along z in thin slices
    double col_wmin_ = 1.0;
    DevBuf<int32_t> cell_key_, cell_count_, cell_start_, cell_fill_, bucket_, col_start_;
    // exclusions
    DevBuf<int32_t> ex_start_, ex_j_;
    DevBuf<uint8_t> ex_bits_;
    // charged-pair list
    DevBuf<int32_t> chg_idx_, chg_key_, chg_count_, chg_start_, chg_fill_;
    DevBuf<float4> chg_sorted_;  // charged beads by cell: x, y, z, index bits
    DevBuf<int32_t> chg_rows_, chg_len_, chg_stats_;  // rows, row lengths, {longest, entries}
    DevBuf<int32_t> ex_csr_;  // per-bead start of its exclusion row (n + 1)
    // bonded
    DevBuf<BondTerm> bonds_;
    DevBuf<AngleTerm> angles_;
    DevBuf<DihedralTerm> dihedrals_;
    DevBuf<FlaTable> fla_;
    DevBuf<FldTable> fld_;
    // misc
    DevBuf<double> energy_;           // kNumSlots
    DevBuf<int32_t> flags_;           // ListFlags bits
    DevBuf<unsigned long long> step_base_;
    DevBuf<double> ke_;
    // snapshot for retries
    DevBuf<double> sx_, sy_, sz_;
    DevBuf<float> svx_, svy_, svz_;
    DevBuf<unsigned long long> sstep_;
    int32_t* h_flags_ = nullptr;  // pinned
};

// Many independent systems, each advanced inside one CTA's shared memory.
class BatchEngine;

}  // namespace ocm
