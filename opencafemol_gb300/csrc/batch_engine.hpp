// batch_engine.hpp - many independent systems advanced by one persistent
// kernel per chunk of steps.  Each CTA claims a system from a work queue
// (largest first), pulls its state into shared memory, runs the chunk
// there (Verlet lists, pair units, chain-local and gathered bonded terms,
// Langevin update) and writes the state back.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <vector>

#include "engine.hpp"
#include "host_system.hpp"

namespace ocm {

// Status of a system in the batch (BatchSys::status).
constexpr int kBatchStatusBlownUp = 1;  // non-finite or out-of-range force, velocity or position

// Device record of one admitted system.

struct BatchSys {
    long long bead_off;    // offset into the bead arena
    long long blob_off;    // byte offset of the static blob
    long long list_off;    // offset (entries) of the neighbour-list region
    int n, nt;             // beads, 32-bead clusters
    int n_bonds, n_angles, n_dih;
    int off_p0, off_p1, off_lab, off_invm;   // byte offsets inside the blob
    // Compact bonded records, the FLA/FLD tables and the chain / gather
    // indices, one contiguous region [off_bonded, off_bonded + bonded_bytes)
    // that the kernel stages into shared memory when it fits; section
    // offsets are relative to it.
    int off_bonded, bonded_bytes;
    int rb_p, rb_ij, ra_ij, ra_k, rd, rgd, rfla, rfld;
    int rcb, rca, rcd, rgs, rgl;
    int off_ex_start, off_ex;                // exclusion CSR (j | bits << 24)
    int maxn;              // neighbour-list entries per bead
    int active;
    int overflow;          // set by the kernel when a list did not fit
    int builds;            // list builds in the last chunk
    int status;            // kBatchStatus*: set by the kernel, the system stops advancing
    int eval_status;       // the same check on the last single evaluation
    float skin;
    PairConsts pc;
    LangevinConsts lc;
    unsigned long long steps_done, steps_target;
};

// First-fit range allocator (units are arbitrary).
class RangeAllocator {
  public:
    explicit RangeAllocator(int64_t cap = 0) { reset(cap); }
    void reset(int64_t cap) {
        cap_ = cap;
        free_.clear();
        if (cap > 0) free_[0] = cap;
    }
    int64_t alloc(int64_t size, int64_t align = 1);  // -1 when full
    void release(int64_t off, int64_t size);
    int64_t capacity() const { return cap_; }
  private:
    int64_t cap_ = 0;
    std::map<int64_t, int64_t> free_;  // offset -> size
};

class BatchEngine {
  public:
    BatchEngine(int device, int64_t max_systems, int64_t max_beads, int32_t max_beads_per_system);
    ~BatchEngine();
    static int64_t footprint(const SystemDesc& d);
    // steps_done > 0 resumes a trajectory: the step counter (and with it
    // the Langevin noise stream) continues from there.
    int64_t admit(const SystemDesc& d, const double* pos, const double* vel, double T,
                  double friction, double dt, int32_t seed, int64_t n_steps, int64_t steps_done = 0);
    int32_t slot_status(int64_t slot);
    // Device-to-device state exchange of one slot with buffers of the same
    // device (the plain context's one-system fast path): positions (FP64
    // SoA), velocities (FP32 SoA), the step counter and the step target.
    // Both wait for the batch's stream; the copies are complete on return.
    void load_state_device(int64_t slot, const double* x, const double* y, const double* z, const float* vx,
                           const float* vy, const float* vz, uint64_t steps_done, uint64_t steps_target);
    void store_state_device(int64_t slot, double* x, double* y, double* z, float* vx, float* vy, float* vz);
    void run(int32_t steps_per_launch, bool sync);
    void finished(int64_t* slots, int64_t cap, int64_t* n_out);
    void get_positions(int64_t slot, double* xyz);
    void get_velocities(int64_t slot, double* v);
    int64_t steps_done(int64_t slot);
    void get_state(int64_t slot, uint32_t groups, double* forces, double* energies);
    void retire(int64_t slot);
    void active(int64_t* n_active, int64_t* beads);
    double last_run_ms();
    void set_threads(int threads);  // 256/512/1024 (autotuner)
    void set_list_smem(int kib);    // -1 = all that fits (autotuner)
    // Balanced launches (the serving loop): the costliest resident system
    // does steps_per_launch steps, the others proportionally more.
    void set_balanced(bool on) { balanced_ = on; }
    // A CTA splits into two groups of half its threads, each with half of
    // its shared memory and its own systems, once the systems left are of at
    // most `beads` beads (0: never; capped so a system fits its half).
    void set_split(int beads);
    int split() const { return split_beads_; }
    void slot_stats(int64_t slot, int32_t* builds, int32_t* capacity);
    void set_positions_many(int64_t n, const int64_t* slots, const double* xyz, const double* v);
    void get_positions_many(int64_t n, const int64_t* slots, double* xyz);
    // Same result without allocating device memory (fixed per-device scratch).
    void get_positions_many_noalloc(int64_t n, const int64_t* slots, double* xyz);
    int threads() const { return threads_; }

  private:
    struct Slot {
        bool used = false;
        int64_t bead_off = 0, n = 0;
        int64_t blob_off = 0, blob_size = 0;
        uint64_t steps_target = 0, steps_done = 0;
        double cost = 0;
        int terms = 0;
        bool labels = false;
        int slot_group[kNumSlots];
        int64_t list_off = 0, list_size = 0;
        int maxn = 0;
        bool failed = false;  // blew up: no longer advanced
    };
    void grow_lists();
    void sync_steps();
    void launch(bool integrate, bool energy, int k, const std::vector<int32_t>& order,
                cudaStream_t s, const std::vector<int32_t>* order_k = nullptr);
    // Estimated time of one MD step of an n-bead system (arbitrary units):
    // the kernel's per-step time grows with n, with a floor set by the
    // per-step barriers of small systems.
    static double step_cost(int64_t n) { return (double)std::max<int64_t>(n, 150); }
    size_t smem_bytes(int nmax, bool general) const;

    int device_;
    int64_t max_systems_, max_beads_;
    int nmax_;
    int threads_ = 512;       // measured best on the 512-replica mix
    int list_smem_kib_ = 96;
    int num_sms_ = 0;
    cudaStream_t stream_ = nullptr, copy_stream_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr, ev_copy_ = nullptr;
    bool ran_ = false;
    std::vector<Slot> slots_;
    RangeAllocator beads_, blob_, list_alloc_;
    DevBuf<double> x_, y_, z_;
    DevBuf<float> vx_, vy_, vz_;
    DevBuf<unsigned char> blob_dev_;
    DevBuf<uint16_t> lists_;
    int* h_overflow_ = nullptr;  // pinned copy of the records' overflow flags
    int* h_status_ = nullptr;    // pinned copy of the records' status words
    int* h_check_ = nullptr;     // pinned: non-finite values found by the upload check
    DevBuf<int> check_;          // the device side of that flag
    DevBuf<BatchSys> sys_;
    DevBuf<int32_t> order_, order_k_, head_;
    bool balanced_ = false;
    int split_beads_ = 512;   // CTA split at systems of at most this many beads (0: never)
    DevBuf<double> energy_;
    DevBuf<float> forces_;
    // staging of the many-slot state copies (grown on demand)
    DevBuf<long long> seg_bead_, seg_off_;
    DevBuf<int> seg_n_;
    std::vector<long long> seg_bead_h_, seg_off_h_;  // host copies of the segment table on the device
    std::vector<int> seg_cnt_h_;
    void upload_segments(int64_t n, const std::vector<long long>& bead, const std::vector<long long>& off,
                         const std::vector<int>& cnt);
    DevBuf<double> stage_;
    std::vector<BatchSys> sys_host_;
};

}  // namespace ocm
