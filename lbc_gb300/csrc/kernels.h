// kernels.h -- host-side launchers of the device kernels (internal header).
#pragma once
#include <cuda_runtime.h>

#include "lbm_device.cuh"

namespace lbm {

enum StoreKind : int { STORE_F64 = 0, STORE_F32 = 1, STORE_F16 = 2 };

struct Wt { double w[9]; };

struct CollideParams {
    int Nx, Ny, pitch;
    long long plane;
    double *f;                       // SoA planes (FP64, or shifted FP32/FP16 as void data)
    const uint16_t *flags;           // solid bit, or null
    const double *rho, *ux, *uy;     // stored fields, dense [Ny * Nx]
    const double *omega;
    double omega0;
    int has_force;
    double Fx, Fy;
    double w[9];
    // Shifted storage only: the stored fields are the moments of the
    // populations (state left by a previous run), so recompute them from the
    // populations in the fused step's own arithmetic.
    int from_pops;
    // FP64 storage: collide as the fused multiply-add step does (collide_fma
    // off the BC-written nodes), so that run(a) + run(b) = run(a + b).
    int fma;
};

// Collision that reads lbc's AoS populations where they are (host memory the
// device can reach, or device memory), writes the post-collision values back in
// place and into the device SoA planes.
struct CollideAosParams {
    int Nx, Ny, pitch;
    long long plane;
    double *f_aos;                   // [Ny][Nx][9], read and written in place
    double *soa;                     // device planes (FP64)
    const uint16_t *flags;
    const double *rho, *ux, *uy;     // stored fields [Ny][Nx] (host or device)
    const double *omega;
    double omega0;
    int has_force;
    double Fx, Fy;
    double w[9];
};

// Arguments of lbc's standalone functions on device copies of lbc's AoS arrays.
struct AosArgs {
    int Nx, Ny, px, py;
    double *f, *fnew;                // [Ny][Nx][9]
    double *rho, *u, *v;             // [Ny][Nx]
    const double *omega, *phi;
    const int *mask;
    double Fx, Fy;
    double w[9];
    double *partials;                // reductions
    unsigned int *ticket;
    double *out2;
};

// One case's force (k_force_reduce): the sum of its segment partials
// partials[2 t .. 2 t + 1], t in [t0, t1), in that order, into out[0..1] (and
// the next slot of the history ring, when there is one).
struct ForceSlot {
    int t0, t1;
    const double *partials;
    double *out;
    double *hist;
    unsigned long long *hist_count;
    int hist_cap;
    int pad;
};

enum AosOp : int { AOS_COLLISION, AOS_STREAMING, AOS_MOMENTS, AOS_BOUNCE_BACK, AOS_IBB, AOS_MEM };

// Parameters of the shifted-storage (FP32 / FP16) fused step.
struct FastStepParams {
    StepParams s;
    float wf[9];
    float omega0f;
    float Fxf, Fyf, hFxf, hFyf;   // FP32 copies (no per-thread FP64 conversions)
    // odd-part coefficients of the equilibrium: h1 = fl(3 w1), h5 = (1 - 2 h1) / 4
    // (2 h1 + 4 h5 = 1 holds exactly); the same bits as shifted_h() on the device
    float h1f, h5f;
};

// Up to kStageGroupMax Boundary entries that touch disjoint band nodes, in one
// launch (blockIdx.y = member), passed by value. Members finish the nodes
// their entry writes last with `fin`; nfs > 0 adds one row of blocks
// (blockIdx.y = n) whose first warp reduces the case's force slot *fs.
constexpr int kStageGroupMax = 6;
struct StageGroup {
    StageParams p[kStageGroupMax];
    int n;
    int max_along;
    FinishParams fin;
    const ForceSlot *fs;
    int nfs;
    int warm;   // FP64: run the instruction-cache warm-up pass (small grids)
};

// Per-step records, one block per task, launched after a step's last kernel:
// probes (density and velocity at chosen nodes, from the populations the step
// left) and impedance-wall traces (the wall's mean p' and v over its active
// nodes, the per-step record lbc's nit case writes, cases/nit/nit.c:262-273).
// Each task's ring holds `cap` steps; *count counts the steps recorded.
enum : int { REC_PROBES = 0, REC_WALL = 1 };
struct RecordTask {
    int kind;
    int n;                       // probes: number of nodes; wall: nodes along the wall
    int cs;                      // batch case index (its step parameters), -1 alone
    int cap;
    const long long *nodes;      // probes: plane offsets
    long long plane;
    const double *imp;           // wall: impedance state [fields][n]
    double *ring;                // probes: [cap][n][3] (rho, ux, uy); wall: [cap][2] (p', v)
    unsigned long long *count;
    double w[9];                 // shifted storage: f = g + w
    double hFx, hFy;             // half the body force: lbc's u = (j + F / 2) / rho
};

namespace launch {
// Records of one step: tasks[0 .. n). Alone: the step's populations are at
// dst. In a batch (spbase set): case cs's are the dst of its step parameters
// for this direction, spbase + (2 cs + sel) * spstride bytes.
// collided: the step ended with a collision (Guo's forcing then added F to the
// momentum, so u = (j - F / 2) / rho); a run's last step leaves pre-collision
// populations (u = (j + F / 2) / rho, as lbc's moments).
cudaError_t record(const RecordTask *tasks, int n, int store, const void *dst, const char *spbase, int spstride,
                   int sel, bool collided, cudaStream_t s);
// FP64 (kernels_exact.cu): lbc's rounding sequence, or with fma set the
// fused multiply-add arithmetic (moments_fma / collide_fma)
cudaError_t step_exact(const StepParams &p, bool flags, bool collide, dim3 block, cudaStream_t s,
                       bool fma = false);
// collide: the finish of fused members applies the collision (false only in
// the final step of a run, which leaves pre-collision populations).
// after_bulk (here, stage_batch and force_reduce): the previous launch in s is
// a bulk step kernel; the launch overlaps its tail (pdl.cuh).
cudaError_t stage_group(const StageGroup &g, int store, bool collide, bool after_bulk, cudaStream_t s);
cudaError_t collide_exact(const CollideParams &p, cudaStream_t s);
cudaError_t collide_aos_exact(const CollideAosParams &p, cudaStream_t s);
cudaError_t aos_to_soa(const double *aos, void *soa, int store, int Nx, int Ny, int pitch,
                       long long plane, const double w[9], cudaStream_t s);
cudaError_t soa_to_aos(const void *soa, double *aos, int store, int Nx, int Ny, int pitch,
                       long long plane, const double w[9], cudaStream_t s);
cudaError_t seed_band(const int2 *nodes, const int *slots, int n, int Nx, const double *rho,
                      const double *ux, const double *uy, double *bandm, int nslots,
                      cudaStream_t s);
cudaError_t aos_op(int op, const AosArgs &a, cudaStream_t s);
unsigned aos_mem_blocks(int Nx, int Ny);
cudaError_t aos_bc(const AosArgs &a, int kind, int index, int along, const double *val1,
                   const double *val2, cudaStream_t s);
cudaError_t mei_init(const AosArgs &a, double rho0, cudaStream_t s);
cudaError_t mei_iter(const AosArgs &a, double rho0, unsigned long long *maxbits, cudaStream_t s);
// lbc's sponge_layer omega field, [Ny][Nx] into omega (device or device-reachable memory)
cudaError_t sponge(int Nx, int Ny, double dx, double xc, double yc, double r_inner, double r_outer,
                   double tau_base, double incr_tau, double exp_coeff, double *omega, cudaStream_t s);
// blocks x 256 threads, each 8 x iters dependent DFMA (lbm_gpu_fp64_rate)
cudaError_t fp64_rate(int blocks, int iters, double *sink, cudaStream_t s);

// batches of cases (tile list = int4 {case, x0, y0, case has wall links})
// Tiles of 2^tws x 2^(8 - tws) nodes, tws in [5, 8].
cudaError_t step_batch_exact(const StepParams *sp, const int4 *tiles, int ntiles,
                             int sel, int tws, int grid, cudaStream_t s, bool fma = false);
int step_batch_exact_grid();
// One level of a batch's Boundary lists (n entries): block b steps points
// blocks[b].y .. + kStageBatchPoints(F64) - 1 of entry blocks[b].x, or, for
// blocks[b].x >= n, reduces force slot fs[blocks[b].x - n].
// warm: FP64 only, run the edge threads' instruction-cache warm-up pass.
constexpr int kStageBatchPoints = 64, kStageBatchPointsF64 = 32;
cudaError_t stage_batch(const StageParams *list, int n, const int2 *blocks, int nblocks,
                        int store, int sel, const ForceSlot *fs, bool after_bulk, bool warm, cudaStream_t s);
cudaError_t force_reduce(const ForceSlot *slots, int n, bool after_bulk, cudaStream_t s);

// shifted storage (kernels_shifted.cu)
cudaError_t step_shifted(const FastStepParams &p, int store, bool flags, bool collide, dim3 block,
                         cudaStream_t s, bool after = false);
// The special nodes of a case (nodes[0 .. n)) on the per-node path; flags: the
// case has a flag word. after_bulk: the programmatic follower of the kernel
// before it (a case alone launches it first, without the attribute, and the
// clean pairs as its follower: step_shifted's after).
cudaError_t special_shifted(const FastStepParams &p, const int2 *nodes, int n, int store, bool flags, bool collide,
                            bool after_bulk, cudaStream_t s);
// The special nodes of a batch: nodes[q] = (case, i, j, chunk), n a multiple
// of 32 (each case's list padded to 32 entries, i = -1); links: some case has
// cut-link records.
cudaError_t special_batch_shifted(const FastStepParams *sp, const int4 *nodes, int n, int sel,
                                  int store, bool wide, bool force, bool links, bool after, cudaStream_t s);
// Edge BCs of shifted storage in FP32 (launch::stage_group / stage_batch dispatch here).
cudaError_t stage_group_shifted(const StageGroup &g, int store, bool collide, bool after_bulk, cudaStream_t s);
cudaError_t stage_batch_shifted(const StageParams *list, int n, const int2 *blocks, int nblocks,
                                int store, int sel, const ForceSlot *fs, bool after_bulk, cudaStream_t s);
cudaError_t collide_shifted(const CollideParams &p, int store, cudaStream_t s);
// wide: some case has 9 * plane >= 2^31 elements (64-bit element offsets).
// force: some case has a body force (the forced kernel form serves all cases).
// all_flags: every case has a flag word (the flag-free pair form is left out).
cudaError_t step_batch_shifted(const FastStepParams *sp, const int4 *tiles,
                               int ntiles, int sel, int tws, int store, bool wide, bool force, bool all_flags,
                               int grid, cudaStream_t s);
int step_batch_shifted_grid(int store);
int sm_count();
}  // namespace launch

}  // namespace lbm
