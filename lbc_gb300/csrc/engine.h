// engine.h -- host-side solver of the GB300 D2Q9 engine (internal header).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "kernels.h"
#include "lbm_device.cuh"

namespace lbm {

void set_error(const std::string &msg);
const char *last_error();
bool check_cuda(cudaError_t e, const char *what);
// Stream-ordered device allocation from the device's default pool (set up to
// retain freed memory), freed with cudaFreeAsync on the owner's stream.
bool device_alloc(void **q, size_t bytes, cudaStream_t s);
void use_retaining_pool();

// Rows of lbc's FP64 AoS arrays (72 B per node) that set_state / get_state
// convert per chunk: 64 MiB of staging at most (one row when a row is larger),
// so that staging costs no per-node device memory.
inline int staging_rows(int Nx, int Ny) {
    const long long row = 72LL * Nx;
    const long long r = (64LL << 20) / row;
    return (int)std::max(1LL, std::min<long long>(Ny, r));
}

// One entry of the Boundary list, resolved to a device BC kind.
struct BCEntry {
    int kind;      // BCKind
    int index;
    const double *val1, *val2;  // host arrays (lbc: length Ny for columns, Nx for rows)
};

// Everything a case needs besides its populations (what main_lbm receives).
struct CaseDesc {
    int Nx = 0, Ny = 0;
    double w[9];
    const int *mask = nullptr;
    const double *omega = nullptr;
    const double *phi = nullptr;
    int use_ibb = 0;
    const double *wall_u = nullptr, *wall_v = nullptr;
    int px = 0, py = 0;
    double Fx = 0.0, Fy = 0.0;
    std::vector<BCEntry> bcs;
    int store = STORE_F64;
    // FP64 storage only: step with the fused multiply-add arithmetic
    // (moments_fma / collide_fma), lbc's results to rounding instead of bit
    // for bit; needs lbc's weight symmetry (w1..w4 equal, w5..w8 equal).
    bool fma64 = false;
};

// The public storage codes (lbm_gpu.h): LBM_GPU_F64_FMA is FP64 storage with
// the fused multiply-add step. False for an unknown code.
inline bool storage_to_desc(int storage, CaseDesc &d) {
    if (storage < 0 || storage > 3) return false;
    d.store = storage == 3 ? STORE_F64 : storage;
    d.fma64 = storage == 3;
    return true;
}

struct Stage {
    int kind, index, along;
    int entry;                  // position in the Boundary list
    // per point t: the BC's node is fluid (every point of a periodic entry);
    // a solid node's point writes nothing, so batches launch no block whose
    // points are all solid
    std::vector<uint8_t> open;
    double *d_val1 = nullptr, *d_val2 = nullptr;
    // impedance wall (bottom regularized entries only)
    double *d_imp = nullptr;

    int imp_nf = 0;
    double imp_alpha = 0.0;
    double imp_wcos = 1.0, imp_wsin = 0.0;
    int imp_windowed = 0;
    double imp_cos[8] = {1, 1, 1, 1, 1, 1, 1, 1}, imp_sin[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    // the wall's per-step trace (mean p', v), when enabled
    double *d_trace = nullptr;
    unsigned long long *trace_count = nullptr;
    int trace_cap = 0;
    unsigned long long trace_written = 0;
};

// Most probes a solver records (one block of a record launch walks them).
constexpr int kMaxProbes = 4096;

// Zero-order-hold update of m v' + R v + K x = p over one lattice step:
// (x, v) <- A (x, v) + b p. Returns false unless m > 0 and K > 0.
bool msd_zoh(double R, double m, double K, double A[4], double b[2]);

class Solver {
  public:
    explicit Solver(const CaseDesc &d);
    ~Solver();
    bool ok() const { return ok_; }

    // Host arrays in lbc's layout. set_state makes buf[cur] = f and the other
    // buffer = f_new, and takes rho/u/v as the stored fields of the next step.
    bool set_state(const double *f, const double *f_new, const double *rho, const double *u,
                   const double *v, bool fnew_needed = true);
    bool get_state(double *f, double *f_new, double *rho, double *u, double *v);
    bool get_fields(double *rho, double *u, double *v);
    // One lbc main_lbm call on the caller's arrays when the device can reach
    // them directly (page-locked, or pageable over NVLink-C2C address
    // translation): the kernels read and write the host arrays themselves.
    bool dropin_step_direct(double *f, double *f_new, double *rho, double *u, double *v);
    // Whether the old content of f_new can reach the results (solid nodes, or
    // populations pulled from off a non-periodic edge).
    bool needs_old_dst() const { return needs_old_dst_; }
    // Copies val1/val2 of Boundary entry `entry` to the device (null keeps the
    // current values); the caller's arrays are not kept.
    bool set_bc_values(int entry, const double *val1, const double *val2);
    bool upload_all_bc_values();
    int bc_count() const { return (int)d_.bcs.size(); }
    // n time steps, each equivalent to one main_lbm call plus the caller's swap.
    bool run(int nsteps);
    bool forces(double *Fx, double *Fy);  // MEM force of the last step
    // Per-step force record (lbm_gpu_force_history).
    bool enable_force_history(int capacity);
    int force_history(double *out, int max_steps);
    // Appends (append) or writes the force records of the steps not written
    // yet; returns their count, or -1. -2: some steps left the ring unwritten.
    long long write_force_records(const char *path, double dt, double cf, bool append);

    int Nx() const { return d_.Nx; }
    int Ny() const { return d_.Ny; }
    int store() const { return d_.store; }
    bool fma64() const { return d_.fma64; }
    // The public storage code (lbm_gpu.h), LBM_GPU_F64_FMA included.
    int storage_code() const { return d_.fma64 ? 3 : d_.store; }
    cudaStream_t stream() const { return stream_; }
    size_t device_bytes() const { return dev_bytes_; }
    bool has_flags() const { return has_flags_; }
    int nstages() const { return (int)stages_.size(); }
    int pitch() const { return pitch_; }
    long long plane() const { return plane_; }
    void *buffer(int b) const { return buf_[b]; }
    int current() const { return cur_; }
    long long steps_done() const { return steps_done_; }
    // Kernel launches per time step inside the loop (for launch counting).
    int launches_per_step() const {
        const int bulk = 1 + (special_launch() ? 1 : 0);
        const int rec = rec_host_.empty() ? 0 : 1;
        // (the loop's steps reduce the wall force only for a force history)
        if (groups_.empty()) return bulk + (has_mem_ && hist_cap_ > 0 ? 1 : 0) + rec;
        return bulk + (int)groups_.size() + rec;
    }
    // Shifted storage: the nodes the clean-pair kernels leave to the
    // special-node kernel (row-major; both nodes of a pair with a special
    // node, and an odd last column). Launched on its own for grids with a
    // flag word; in batches for every case.
    const std::vector<int2> &special_nodes() const { return special_host_; }
    bool special_launch() const { return d_.store != STORE_F64 && has_flags_ && nspecial_ > 0; }
    bool set_block(dim3 b);
    dim3 block() const { return block_; }
    // Launch-shape tuning (tune.h). mode 1: take the cached block for this
    // case's key, else time the candidate blocks on the first steps of the
    // next run that has enough of them and keep the fastest. mode 0: off.
    void set_autotune(int mode);
    int autotune_mode() const { return tune_mode_; }
    bool tuned() const { return tuned_; }
    float tuned_us() const { return tuned_us_; }
    std::string tune_key() const;

    // Pieces used by Batch: parameters of one step in a given direction, the
    // first-step collision and the final (pre-collision, moments) step.
    StepParams step_params(int src, int dst, bool write_macro, int bparity) const;
    FastStepParams fast_params(const StepParams &p) const;
    StageParams stage_params(const Stage &st, int src, int bparity) const;
    FinishParams finish_params(int dst, bool write_macro, int bparity) const;
    const std::vector<Stage> &stages() const { return stages_; }
    // Consecutive stages that share one launch (indices into stages()).
    const std::vector<std::vector<int>> &stage_groups() const { return groups_; }
    bool has_mem() const { return has_mem_; }
    bool has_links() const { return has_links_; }
    bool has_force() const { return d_.Fx != 0.0 || d_.Fy != 0.0; }
    // 1 for fluid nodes with at least one solid pull source (wall link), [Ny][Nx].
    const std::vector<uint8_t> &link_nodes() const { return link_node_; }
    int parity() const { return parity_; }
    double *mem_out() const { return d_mem_out_; }
    double *hist() const { return d_hist_; }
    unsigned long long *hist_count() const { return hist_count_ptr_; }
    int hist_cap() const { return hist_cap_; }
    // Where this case's force is reduced from and written to.
    ForceSlot force_slot() const;
    // Tiles of 2^tws x 2^(8 - tws) threads covering this case for the batched
    // kernel (cached per shape).
    const std::vector<int4> &tiles(int tws) const;
    // Impedance wall on Boundary entry `entry` (velocity_bottom_regularized):
    // per node R, m, K (m <= 0: keep the entry's own val2), nf <= 8 DFT
    // frequencies (rad / step), reference density for p' and the rate of its
    // running average (0: fixed).
    bool set_impedance(int entry, const double *R, const double *m, const double *K, int nf,
                       const double *omegas, double rho_ref, double alpha, int window);
    // out[((t * nf) + f) * 4 + {0,1,2,3}] = (P re, P im, V re, V im); state[t*2+{0,1}] = (x, v)
    bool impedance_readback(int entry, double *out, double *state);
    // Population checkpoint (io.cpp): everything a continued run reads, so
    // that save after run(a), load into a solver of the same case (with the
    // same impedance-wall setup and force-history capacity) and run(b) equal
    // run(a + b) bit for bit.
    bool checkpoint_save(const char *path);
    bool checkpoint_load(const char *path);
    // Device-packed VTK of the stored fields (io.cpp): lbc's
    // write_vtk_binary_2D bytes, packed on the device and written by a host
    // thread while the solver keeps stepping; finished by vtk_wait().
    bool write_vtk(const char *path, double dx, double cu, double crho);
    bool vtk_wait();
    // Probes: density and velocity (rho, ux, uy) at n nodes after every step,
    // in a device ring of `capacity` steps (n = 0 removes them).
    bool set_probes(int n, const int *i, const int *j, int capacity);
    // Copies up to max_steps records, oldest first: out[(t n + q) 3 + {0,1,2}].
    int probe_history(double *out, int max_steps);
    // The impedance wall's per-step trace on Boundary entry `entry`.
    bool enable_impedance_trace(int entry, int capacity);
    long long write_impedance_trace(int entry, const char *path, double dt, double cp, double cu, bool append);
    // The record tasks of this solver (probes, wall traces) for a batch.
    const std::vector<RecordTask> &record_tasks() const { return rec_host_; }
    bool begin_steps(cudaStream_t s);
    bool end_steps(cudaStream_t s);
    void advance(int nsteps);
    void add_steps(long long n) { steps_done_ += n; }

  private:
    bool build_geometry();
    bool alloc();
    bool launch_step(int src, int dst, bool collide, bool write_macro, int bparity,
                     cudaStream_t s = nullptr);
    bool launch_step_kernels(int src, int dst, bool collide, bool write_macro, int bparity, cudaStream_t s);
    bool upload_records();
    std::vector<RecordTask> rec_host_;
    RecordTask *d_rec_ = nullptr;
    int rec_cap_ = 0;
    long long *d_probe_nodes_ = nullptr;
    double *d_probe_ring_ = nullptr;
    unsigned long long *probe_count_ = nullptr;
    int nprobes_ = 0, probe_cap_ = 0;
    bool launch_collide(int b, cudaStream_t s = nullptr);
    bool capture_pair();
    bool trial_step();
    int tune_online(int avail);
    int tune_mode_ = 0;
    bool tuned_ = false;
    float tuned_us_ = 0.f;
    template <class T> bool dalloc(T **p, size_t count);

    CaseDesc d_;
    bool ok_ = false;
    cudaStream_t stream_ = nullptr;
    int pitch_ = 0;
    long long plane_ = 0;
    size_t esize_ = 8;
    void *buf_[2] = {nullptr, nullptr};
    int cur_ = 0;
    int parity_ = 0;
    bool has_flags_ = false, has_links_ = false, has_mem_ = false;
    uint16_t *d_flags_ = nullptr;
    int *d_link_off_ = nullptr;
    Link *d_links_ = nullptr;
    double *d_omega_ = nullptr;
    double omega0_ = 1.0;
    int *d_colbase_ = nullptr, *d_rowbase_ = nullptr;
    int nslots_ = 0;
    double *d_bandf_ = nullptr;  // FP64 storage
    float *d_bandg_ = nullptr;   // shifted storage
    double *d_bandm_[2] = {nullptr, nullptr};
    int2 *d_seed_nodes_ = nullptr;
    int *d_seed_slots_ = nullptr;
    int nseed_ = 0;
    double *d_rho_ = nullptr, *d_ux_ = nullptr, *d_uy_ = nullptr;
    double *d_partials_ = nullptr;
    double *d_mem_out_ = nullptr;
    double *d_hist_ = nullptr;
    int hist_cap_ = 0;
    unsigned long long *hist_count_ptr_ = nullptr;
    unsigned long long hist_written_ = 0;  // steps whose force record is in a file
    double *d_stage_ = nullptr;  // AoS staging: staging_rows() rows of FP64 AoS
    int stage_rows_ = 1;
    std::vector<Stage> stages_;
    std::vector<std::vector<int>> groups_;
    template <class Solid>
    bool group_stages(const Solid &solid, const std::vector<int> &colbase, const std::vector<int> &rowbase);
    // Per band slot: the last stage (index into stages_) that writes the node, -1 for none.
    std::vector<short> last_host_;
    short *d_last_ = nullptr;
    dim3 block_{64, 4, 1};
    cudaGraphExec_t pair_exec_ = nullptr;
    int pair_cur_ = -1, pair_parity_ = -1;
    bool graph_valid_ = false;
    size_t dev_bytes_ = 0;
    long long steps_done_ = 0;
    std::vector<void *> allocs_;
    bool needs_old_dst_ = true;
    bool fields_are_moments_ = false;  // stored rho/u/v are the moments of the current populations
    std::vector<uint8_t> link_node_;
    mutable std::map<int, std::vector<int4>> tile_cache_;
    // VTK packing: device staging, pinned host copy, the writer thread
    unsigned char *d_vtk_ = nullptr, *h_vtk_ = nullptr;
    size_t vtk_bytes_ = 0;
    cudaEvent_t vtk_ev_ = nullptr;
    std::thread *vtk_thread_ = nullptr;
    bool vtk_ok_ = true;
    std::string vtk_err_;
    int *d_seg_slot_ = nullptr;     // per 32-node row segment (FP64) or 32-entry special-list chunk: force slot or -1
    std::vector<int2> special_host_;
    uint32_t *d_seg_clean_ = nullptr;
    int seg_words_ = 0;
    int2 *d_special_ = nullptr;
    int nspecial_ = 0;
    int nlink_segs_ = 0;
    ForceSlot *d_force_slot_ = nullptr;
    bool compute_segment_slots();
    bool upload_force_slot();
    double *macro_out_[3] = {nullptr, nullptr, nullptr};  // moments written here when set
};

// Many independent cases of one storage type advanced together: per step one
// persistent bulk kernel over the flattened tile list of all cases (shifted
// storage: clean node pairs, then one launch over every case's special nodes),
// then one launch per stage level (the l-th stage group of every case) whose
// threads also finish the nodes their entry wrote last; the first level's
// launch also reduces every case's force. The steps between the per-case
// first collision and final step run from a captured two-step graph. Each
// case ends exactly as Solver::run(n) would leave it.
class Batch {
  public:
    explicit Batch(const std::vector<Solver *> &cases);
    ~Batch();
    bool ok() const { return ok_; }
    bool run(int nsteps);
    int ncases() const { return (int)cases_.size(); }
    long long nodes() const { return nodes_; }
    int launches_per_step() const { return launches_per_step_; }
    cudaStream_t stream() const { return stream_; }

    // Tile shape of the bulk kernel: 2^tws x 2^(8 - tws) nodes, tws in [5, 8].
    int tile_shift() const { return tws_; }
    bool set_tile_shift(int tws) { return tws == tws_ || build_tiles(tws); }
    // Tile-shape tuning, as Solver::set_autotune (the key is the batch's
    // composition: every case's grid and geometry class).
    void set_autotune(int mode);
    bool tuned() const { return tuned_; }
    float tuned_us() const { return tuned_us_; }
    std::string tune_key() const;

  private:
    bool build();
    bool build_tiles(int tws);
    std::vector<int4> make_tiles(int tws) const;
    bool upload_tiles(const std::vector<int4> &tiles, int4 **d);
    void install_tiles(int4 *d, int n, int tws, bool free_old);
    int tune_online(int avail_pairs);
    int tune_mode_ = 0;
    bool tuned_ = false;
    float tuned_us_ = 0.f;
    bool launch_batched(int sel);
    bool capture_pair();

    std::vector<Solver *> cases_;
    int store_ = STORE_F64;
    bool ok_ = false;
    cudaStream_t stream_ = nullptr;
    long long nodes_ = 0;
    int ntiles_ = 0, grid_ = 0, max_stages_ = 0, nforce_ = 0;
    int tws_ = 6;
    bool wide_ = false;  // some case needs 64-bit element offsets
    bool any_force_ = false;  // some case has a body force
    bool all_flags_ = true;   // every case has a flag word
    bool any_links_ = false;  // some case has cut-link records
    bool forces_ = true;      // the batched steps reduce wall forces (some case records them)
    int launches_per_step_ = 0;
    void *d_sp_ = nullptr;         // StepParams or FastStepParams [2 * ncases]
    int4 *d_tiles_ = nullptr;
    std::vector<StageParams *> d_stage_lists_;
    std::vector<int> stage_counts_;
    // per level: the launch's blocks, (entry, first point) or (count + force
    // slot, 0) on the first level
    std::vector<int2 *> d_stage_blocks_;
    std::vector<int> stage_nblocks_;
    FinishParams *d_fin_ = nullptr;
    ForceSlot *d_force_ = nullptr;
    int4 *d_special_ = nullptr;    // (case, i, j, chunk), shifted storage
    int nspecial_ = 0;
    int4 *d_special_nf_ = nullptr; // the same without marked solids (runs that reduce no force)
    int nspecial_nf_ = 0;
    RecordTask *d_rec_ = nullptr;   // every case's probes and wall traces (case index set)
    int nrec_ = 0;
    cudaGraphExec_t pair_exec_ = nullptr;
    std::vector<void *> allocs_;
    // host copies of the per-run parameters (kept until their uploads ran)
    std::vector<StepParams> h_sp_;
    std::vector<FastStepParams> h_fsp_;
    std::vector<FinishParams> h_fin_;
    std::vector<std::vector<StageParams>> h_lists_;
    cudaEvent_t params_ev_ = nullptr;
};

// Maps lbc BC function pointers to device kinds (dropin.cpp).
int bc_kind_of(const void *fn);

}  // namespace lbm
