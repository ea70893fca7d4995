// dropin.cpp -- lbc's C API (include/lbm_core.h, lbm_bc.h, lbm_utils.h) and the
// extended lbm_gpu_* API, on top of the GPU engine.
//
// main_lbm keeps one device solver per case (keyed by the caller's geometry
// pointers and Boundary list); every call uploads the caller's f, f_new and
// rho/u/v, runs one step on the GPU and writes back everything lbc writes:
// post-collision f, f_new, rho/u/v, *L, *D. The other lbc functions run their
// own kernels on device copies of lbc's AoS arrays.
#include <dlfcn.h>
#include <sys/stat.h>
#include <sys/types.h>

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/lbm.h"
#include "../../include/lbm_gpu.h"
#include "engine.h"
#include "tune.h"

using namespace lbm;

namespace {

std::mutex g_mu;

const int kCX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
const int kCY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
const int kOPP[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

bool check_lattice(int Q, const int *cx, const int *cy, const int *opp) {
    if (Q != 9) {
        set_error("only D2Q9 (Q = 9) is supported");
        return false;
    }
    for (int k = 0; k < 9; k++) {
        if ((cx && cx[k] != kCX[k]) || (cy && cy[k] != kCY[k]) || (opp && opp[k] != kOPP[k])) {
            set_error("cx/cy/opp must be lbc's D2Q9 ordering (cases/nit/nit.c:195-202)");
            return false;
        }
    }
    return true;
}

void report(const char *fn) {
    static int printed = 0;
    if (printed < 8) {
        fprintf(stderr, "lbm_gpu: %s failed: %s\n", fn, last_error());
        printed++;
    }
}

// ------------------------------------------------------------------ scratch
// Grow-only device copies of lbc's AoS arrays for the standalone functions.
struct Scratch {
    cudaStream_t s = nullptr;
    std::vector<std::pair<void *, size_t>> bufs;  // by slot
    void *get(int slot, size_t bytes) {
        if ((int)bufs.size() <= slot) bufs.resize(slot + 1, {nullptr, 0});
        auto &b = bufs[slot];
        if (b.second < bytes) {
            if (b.first) cudaFree(b.first);
            b.first = nullptr;
            b.second = 0;
            if (!check_cuda(cudaMalloc(&b.first, bytes), "cudaMalloc scratch")) return nullptr;
            b.second = bytes;
        }
        return b.first;
    }
    bool init() {
        if (s) return true;
        return check_cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    }
};
Scratch g_scr;

enum { SL_F, SL_FNEW, SL_RHO, SL_U, SL_V, SL_OMEGA, SL_PHI, SL_MASK, SL_VAL1, SL_VAL2, SL_PART, SL_TICK, SL_OUT };

bool up(int slot, const void *h, size_t bytes, void **d) {
    *d = g_scr.get(slot, bytes);
    if (!*d) return false;
    return check_cuda(cudaMemcpyAsync(*d, h, bytes, cudaMemcpyHostToDevice, g_scr.s), "H2D");
}
bool down(void *h, const void *d, size_t bytes) {
    return check_cuda(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, g_scr.s), "D2H");
}

// ------------------------------------------------------------------ main_lbm cache
struct DropinKey {
    int Nx, Ny, px, py, use_ibb;
    const void *mask, *omega, *phi;
    double Fx, Fy, w[9];
    std::vector<std::pair<int, int>> bcs;  // kind, index
    bool operator==(const DropinKey &o) const {
        if (Nx != o.Nx || Ny != o.Ny || px != o.px || py != o.py || use_ibb != o.use_ibb ||
            mask != o.mask || omega != o.omega || phi != o.phi || Fx != o.Fx || Fy != o.Fy ||
            bcs != o.bcs)
            return false;
        for (int k = 0; k < 9; k++)
            if (w[k] != o.w[k]) return false;
        return true;
    }
};
struct DropinEntry {
    DropinKey key;
    std::unique_ptr<Solver> solver;
};
std::vector<DropinEntry> g_cache;
bool g_force_staged = false;

// Lazy drop-in (lbm_gpu_dropin_set_lazy): the result of the last main_lbm
// call, still only on the device, and the caller's arrays it belongs to. The
// next call continues from it when the caller has swapped f and f_new (as lbc's
// case mains do, cases/nit/nit.c:309-311); anything else writes it back first.
struct LazyState {
    Solver *s = nullptr;
    DropinKey key;
    double *f = nullptr, *f_new = nullptr, *rho = nullptr, *u = nullptr, *v = nullptr;
};
bool g_lazy = false;
LazyState g_pending;

// Writes a pending lazy result back to the caller's arrays (g_mu held).
bool flush_lazy() {
    if (!g_pending.s) return true;
    const LazyState p = g_pending;
    g_pending = LazyState{};
    return p.s->get_state(p.f_new, p.f, p.rho, p.u, p.v);
}

// g_mu for a drop-in entry point that reads or writes the caller's arrays:
// a pending lazy result reaches them first.
struct EntryLock {
    std::lock_guard<std::mutex> g;
    EntryLock() : g(g_mu) {
        if (!flush_lazy()) report("lbm_gpu_dropin_sync");
    }
};

}  // namespace

// BC kind of an lbc BC function pointer: identity with this library's own
// symbols, else the symbol name (dladdr) of a function with one of lbc's names.
int lbm::bc_kind_of(const void *fn) {
    static const struct { const void *p; int kind; const char *name; } tab[] = {
        {(const void *)&velocity_inlet, BC_VEL_IN_ZH, "velocity_inlet"},
        {(const void *)&velocity_outlet, BC_VEL_OUT_ZH, "velocity_outlet"},
        {(const void *)&velocity_top, BC_VEL_TOP_ZH, "velocity_top"},
        {(const void *)&velocity_bottom, BC_VEL_BOT_ZH, "velocity_bottom"},
        {(const void *)&pressure_inlet, BC_PRES_IN_ZH, "pressure_inlet"},
        {(const void *)&pressure_outlet, BC_PRES_OUT_ZH, "pressure_outlet"},
        {(const void *)&convective_inlet, BC_CONV_IN, "convective_inlet"},
        {(const void *)&convective_outlet, BC_CONV_OUT, "convective_outlet"},
        {(const void *)&periodic_x, BC_PERIODIC_X, "periodic_x"},
        {(const void *)&periodic_y, BC_PERIODIC_Y, "periodic_y"},
        {(const void *)&velocity_inlet_regularized, BC_VEL_IN_REG, "velocity_inlet_regularized"},
        {(const void *)&velocity_outlet_regularized, BC_VEL_OUT_REG, "velocity_outlet_regularized"},
        {(const void *)&velocity_top_regularized, BC_VEL_TOP_REG, "velocity_top_regularized"},
        {(const void *)&velocity_bottom_regularized, BC_VEL_BOT_REG, "velocity_bottom_regularized"},
        {(const void *)&pressure_inlet_regularized, BC_PRES_IN_REG, "pressure_inlet_regularized"},
        {(const void *)&pressure_outlet_regularized, BC_PRES_OUT_REG, "pressure_outlet_regularized"},
        {(const void *)&pressure_top_regularized, BC_PRES_TOP_REG, "pressure_top_regularized"},
        {(const void *)&pressure_bottom_regularized, BC_PRES_BOT_REG, "pressure_bottom_regularized"},
        {(const void *)&velocity_bottom_corrected, BC_VEL_BOT_ZH_FIX, "velocity_bottom_corrected"},
    };
    for (const auto &t : tab)
        if (t.p == fn) return t.kind;
    Dl_info info;
    if (fn && dladdr(fn, &info) && info.dli_sname && info.dli_saddr == fn) {
        for (const auto &t : tab)
            if (std::strcmp(info.dli_sname, t.name) == 0) return t.kind;
    }
    return -1;
}

static bool fill_desc(CaseDesc &d, int Nx, int Ny, const double *w, const double *omega,
                      const int *mask, const Boundary *bnd, int nb, int px, int py, double Fx,
                      double Fy, const double *phi, int use_ibb) {
    d.Nx = Nx;
    d.Ny = Ny;
    for (int k = 0; k < 9; k++) d.w[k] = w[k];
    d.mask = mask;
    d.omega = omega;
    d.phi = phi;
    d.use_ibb = use_ibb;
    d.px = px;
    d.py = py;
    d.Fx = Fx;
    d.Fy = Fy;
    if (use_ibb && !phi) {
        set_error("use_IBB needs phi");
        return false;
    }
    if (nb < 0 || (nb > 0 && !bnd)) {
        set_error("bad boundary list");
        return false;
    }
    for (int b = 0; b < nb; b++) {
        const int kind = bc_kind_of((const void *)bnd[b].apply);
        if (kind < 0) {
            set_error("Boundary entry " + std::to_string(b) +
                      ": apply is not one of lbc's BC functions of this library");
            return false;
        }
        d.bcs.push_back(BCEntry{kind, bnd[b].index, bnd[b].val1, bnd[b].val2});
    }
    return true;
}

static DropinKey make_key(const CaseDesc &d) {
    DropinKey key;
    key.Nx = d.Nx; key.Ny = d.Ny; key.px = d.px; key.py = d.py; key.use_ibb = d.use_ibb;
    key.mask = d.mask; key.omega = d.omega; key.phi = d.use_ibb ? d.phi : nullptr;
    key.Fx = d.Fx; key.Fy = d.Fy;
    for (int k = 0; k < 9; k++) key.w[k] = d.w[k];
    for (const BCEntry &b : d.bcs) key.bcs.push_back({b.kind, b.index});
    return key;
}

static Solver *dropin_solver(const CaseDesc &d) {
    const DropinKey key = make_key(d);
    for (auto &e : g_cache)
        if (e.key == key) return e.solver.get();
    if (g_cache.size() >= 4) g_cache.erase(g_cache.begin());
    std::unique_ptr<Solver> s(new Solver(d));
    if (!s->ok()) return nullptr;
    g_cache.push_back(DropinEntry{key, std::move(s)});
    return g_cache.back().solver.get();
}

extern "C" {

// ------------------------------------------------------------------ main_lbm
// A Boundary list that holds a function of the caller's own (not one of lbc's
// BC functions) cannot run on the device. main_lbm then runs lbc's sequence
// (src/core/main_lbm.c:32-61) from this library's standalone functions, each
// a device kernel over the caller's arrays, and calls every Boundary entry
// through its pointer: lbc's BC functions of this library on the device, the
// caller's own on the host arrays, in list order. The results are lbc's; the
// speed is that of the standalone functions (the arrays cross the host link
// once each way per function). The sequence stops at the first failure.
static bool has_user_bc(const Boundary *bnd, int nb) {
    for (int b = 0; b < nb && bnd; b++)
        if (bnd[b].apply && bc_kind_of((const void *)bnd[b].apply) < 0) return true;
    return false;
}

static void main_lbm_with_user_bcs(int Nx, int Ny, int Q, double *f, double *f_new, double *rho, double *u,
                                   double *v, int cx[], int cy[], double w[], int opp[], double *omega_eff,
                                   int *solid_mask, Boundary boundaries[], int num_boundaries, int isperiodic_x,
                                   int isperiodic_y, double Fx, double Fy, double *L, double *D, double *phi,
                                   int use_IBB) {
    for (int b = 0; b < num_boundaries; b++)
        if (!boundaries[b].apply) {
            set_error("Boundary entry " + std::to_string(b) + ": apply is NULL");
            return report("main_lbm");
        }
    if (use_IBB && !phi) {
        set_error("use_IBB needs phi");
        return report("main_lbm");
    }
    { EntryLock flush; }
    const std::string before = last_error();
    set_error("");
    auto failed = [] { return last_error()[0] != '\0'; };
    double fx = 0.0, fy = 0.0;
    collision(Nx, Ny, Q, f, rho, u, v, omega_eff, solid_mask, cx, cy, w, Fx, Fy);
    if (failed()) return;
    if (use_IBB)
        interpolated_bounce_back(Nx, Ny, Q, f, f_new, solid_mask, phi, opp, cx, cy, isperiodic_x, isperiodic_y);
    else
        bounce_back(Nx, Ny, Q, f, f_new, solid_mask, cx, cy, opp, isperiodic_x, isperiodic_y);
    if (failed()) return;
    compute_force_mem(Nx, Ny, Q, f, f_new, solid_mask, isperiodic_x, isperiodic_y, cx, cy, opp, &fx, &fy);
    if (failed()) return;
    streaming(Nx, Ny, Q, f, f_new, solid_mask, cx, cy, isperiodic_x, isperiodic_y);
    if (failed()) return;
    for (int b = 0; b < num_boundaries; b++) {
        boundaries[b].apply(Nx, Ny, Q, boundaries[b].index, boundaries[b].val1, boundaries[b].val2, f, f_new,
                            rho, u, v, solid_mask, cx, cy, w);
        if (failed()) return;
    }
    compute_macroscopic_fields(Nx, Ny, Q, f_new, solid_mask, cx, cy, rho, u, v, Fx, Fy);
    if (failed()) return;
    if (D) *D = fx;
    if (L) *L = fy;
    set_error(before);
}

void main_lbm(int Nx, int Ny, int Q, double *f, double *f_new, double *rho, double *u, double *v,
              int cx[], int cy[], double w[], int opp[], double *omega_eff, int *solid_mask,
              Boundary boundaries[], int num_boundaries, int isperiodic_x, int isperiodic_y,
              double Fx, double Fy, double *L, double *D, double *phi, int use_IBB) {
    if (num_boundaries > 0 && has_user_bc(boundaries, num_boundaries))
        return main_lbm_with_user_bcs(Nx, Ny, Q, f, f_new, rho, u, v, cx, cy, w, opp, omega_eff, solid_mask,
                                      boundaries, num_boundaries, isperiodic_x, isperiodic_y, Fx, Fy, L, D, phi,
                                      use_IBB);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!check_lattice(Q, cx, cy, opp)) return report("main_lbm");
    CaseDesc d;
    if (!fill_desc(d, Nx, Ny, w, omega_eff, solid_mask, boundaries, num_boundaries, isperiodic_x,
                   isperiodic_y, Fx, Fy, phi, use_IBB))
        return report("main_lbm");
    // Lazy: continue on the device when this call takes the last one's result
    // (f = its f_new, f_new = its f, same fields and case); otherwise write a
    // pending result back before anything else.
    const bool cont = g_lazy && g_pending.s && g_pending.f == f_new && g_pending.f_new == f &&
                      g_pending.rho == rho && g_pending.u == u && g_pending.v == v && g_pending.key == make_key(d);
    if (!cont && !flush_lazy()) return report("main_lbm");
    Solver *s = dropin_solver(d);
    if (!s) return report("main_lbm");
    for (int b = 0; b < num_boundaries; b++)
        if (!s->set_bc_values(b, boundaries[b].val1, boundaries[b].val2)) return report("main_lbm");
    double fx = 0.0, fy = 0.0;
    if (g_lazy) {
        g_pending = LazyState{};
        if ((!cont && !s->set_state(f, f_new, rho, u, v, s->needs_old_dst())) || !s->run(1) ||
            !s->forces(&fx, &fy))
            return report("main_lbm");
        g_pending.s = s;
        g_pending.key = make_key(d);
        g_pending.f = f; g_pending.f_new = f_new;
        g_pending.rho = rho; g_pending.u = u; g_pending.v = v;
        if (D) *D = fx;
        if (L) *L = fy;
        return;
    }
    // GB300: when the device can reach the caller's arrays (page-locked, or any
    // pageable memory through the NVLink-C2C address translation), the kernels
    // stream them directly; otherwise stage them through copies.
    const bool direct = !g_force_staged && lbm_gpu_host_access(f) > 0 &&
                        lbm_gpu_host_access(f_new) > 0 && lbm_gpu_host_access(rho) > 0 &&
                        lbm_gpu_host_access(u) > 0 && lbm_gpu_host_access(v) > 0;
    if (direct) {
        if (!s->dropin_step_direct(f, f_new, rho, u, v) || !s->forces(&fx, &fy)) return report("main_lbm");
    } else if (!s->set_state(f, f_new, rho, u, v, s->needs_old_dst()) || !s->run(1) ||
               !s->get_state(f_new, f, rho, u, v) ||
               !s->forces(&fx, &fy)) {
        return report("main_lbm");
    }
    if (D) *D = fx;
    if (L) *L = fy;
}

// ------------------------------------------------------------------ standalone core functions
static bool aos_begin(AosArgs &a, int Nx, int Ny, int px, int py) {
    std::memset(&a, 0, sizeof a);
    a.Nx = Nx;
    a.Ny = Ny;
    a.px = px;
    a.py = py;
    return g_scr.init();
}

void collision(int Nx, int Ny, int Q, double *f, double *rho, double *u, double *v,
               double *omega_eff, int *solid_mask, int cx[], int cy[], double w[], double Fx,
               double Fy) {
    EntryLock lk;
    AosArgs a;
    const size_t N = (size_t)Nx * Ny;
    if (!check_lattice(Q, cx, cy, nullptr) || !aos_begin(a, Nx, Ny, 0, 0)) return report("collision");
    void *p;
    bool okk = up(SL_F, f, N * 9 * 8, &p); a.f = (double *)p;
    okk = okk && up(SL_RHO, rho, N * 8, &p); a.rho = (double *)p;
    okk = okk && up(SL_U, u, N * 8, &p); a.u = (double *)p;
    okk = okk && up(SL_V, v, N * 8, &p); a.v = (double *)p;
    okk = okk && up(SL_OMEGA, omega_eff, N * 8, &p); a.omega = (double *)p;
    okk = okk && up(SL_MASK, solid_mask, N * 4, &p); a.mask = (int *)p;
    for (int k = 0; k < 9; k++) a.w[k] = w[k];
    a.Fx = Fx; a.Fy = Fy;
    okk = okk && check_cuda(launch::aos_op(AOS_COLLISION, a, g_scr.s), "collision") &&
          down(f, a.f, N * 9 * 8) && check_cuda(cudaStreamSynchronize(g_scr.s), "collision");
    if (!okk) report("collision");
}

void streaming(int Nx, int Ny, int Q, double *f, double *f_new, int *solid_mask, int cx[],
               int cy[], int isperiodic_x, int isperiodic_y) {
    EntryLock lk;
    AosArgs a;
    const size_t N = (size_t)Nx * Ny;
    if (!check_lattice(Q, cx, cy, nullptr) || !aos_begin(a, Nx, Ny, isperiodic_x, isperiodic_y))
        return report("streaming");
    void *p;
    bool okk = up(SL_F, f, N * 9 * 8, &p); a.f = (double *)p;
    okk = okk && up(SL_FNEW, f_new, N * 9 * 8, &p); a.fnew = (double *)p;
    okk = okk && up(SL_MASK, solid_mask, N * 4, &p); a.mask = (int *)p;
    okk = okk && check_cuda(launch::aos_op(AOS_STREAMING, a, g_scr.s), "streaming") &&
          down(f_new, a.fnew, N * 9 * 8) && check_cuda(cudaStreamSynchronize(g_scr.s), "streaming");
    if (!okk) report("streaming");
}

void compute_macroscopic_fields(int Nx, int Ny, int Q, double *f_new, int *solid_mask, int cx[],
                                int cy[], double *rho, double *u, double *v, double Fx, double Fy) {
    EntryLock lk;
    AosArgs a;
    const size_t N = (size_t)Nx * Ny;
    if (!check_lattice(Q, cx, cy, nullptr) || !aos_begin(a, Nx, Ny, 0, 0))
        return report("compute_macroscopic_fields");
    void *p;
    bool okk = up(SL_FNEW, f_new, N * 9 * 8, &p); a.fnew = (double *)p;
    okk = okk && up(SL_MASK, solid_mask, N * 4, &p); a.mask = (int *)p;
    a.rho = (double *)g_scr.get(SL_RHO, N * 8);
    a.u = (double *)g_scr.get(SL_U, N * 8);
    a.v = (double *)g_scr.get(SL_V, N * 8);
    a.Fx = Fx; a.Fy = Fy;
    okk = okk && a.rho && a.u && a.v &&
          check_cuda(launch::aos_op(AOS_MOMENTS, a, g_scr.s), "moments") && down(rho, a.rho, N * 8) &&
          down(u, a.u, N * 8) && down(v, a.v, N * 8) &&
          check_cuda(cudaStreamSynchronize(g_scr.s), "moments");
    if (!okk) report("compute_macroscopic_fields");
}

void compute_force_mem(int Nx, int Ny, int Q, double *f, double *f_new, int *solid_mask,
                       int isperiodic_x, int isperiodic_y, const int cx[], const int cy[],
                       const int opp[], double *Fx, double *Fy) {
    EntryLock lk;
    AosArgs a;
    const size_t N = (size_t)Nx * Ny;
    if (!check_lattice(Q, cx, cy, opp) || !aos_begin(a, Nx, Ny, isperiodic_x, isperiodic_y))
        return report("compute_force_mem");
    void *p;
    bool okk = up(SL_F, f, N * 9 * 8, &p); a.f = (double *)p;
    okk = okk && up(SL_FNEW, f_new, N * 9 * 8, &p); a.fnew = (double *)p;
    okk = okk && up(SL_MASK, solid_mask, N * 4, &p); a.mask = (int *)p;
    const unsigned nb = launch::aos_mem_blocks(Nx, Ny);
    a.partials = (double *)g_scr.get(SL_PART, (size_t)nb * 16);
    a.ticket = (unsigned int *)g_scr.get(SL_TICK, 16);
    a.out2 = (double *)g_scr.get(SL_OUT, 16);
    double h[2] = {0, 0};
    okk = okk && a.partials && a.ticket && a.out2 &&
          check_cuda(cudaMemsetAsync(a.ticket, 0, 4, g_scr.s), "memset") &&
          check_cuda(launch::aos_op(AOS_MEM, a, g_scr.s), "mem") && down(h, a.out2, 16) &&
          check_cuda(cudaStreamSynchronize(g_scr.s), "mem");
    if (!okk) return report("compute_force_mem");
    *Fx = h[0];
    *Fy = h[1];
}

void bounce_back(int Nx, int Ny, int Q, double *f, double *f_new, int *solid_mask, int cx[],
                 int cy[], int opp[], int isperiodic_x, int isperiodic_y) {
    EntryLock lk;
    AosArgs a;
    const size_t N = (size_t)Nx * Ny;
    if (!check_lattice(Q, cx, cy, opp) || !aos_begin(a, Nx, Ny, isperiodic_x, isperiodic_y))
        return report("bounce_back");
    void *p;
    bool okk = up(SL_F, f, N * 9 * 8, &p); a.f = (double *)p;
    okk = okk && up(SL_FNEW, f_new, N * 9 * 8, &p); a.fnew = (double *)p;
    okk = okk && up(SL_MASK, solid_mask, N * 4, &p); a.mask = (int *)p;
    okk = okk && check_cuda(launch::aos_op(AOS_BOUNCE_BACK, a, g_scr.s), "bounce_back") &&
          down(f_new, a.fnew, N * 9 * 8) && check_cuda(cudaStreamSynchronize(g_scr.s), "bounce_back");
    if (!okk) report("bounce_back");
}

void interpolated_bounce_back(int Nx, int Ny, int Q, double *f, double *f_new, int *solid_mask,
                              double *phi, int opp[], int cx[], int cy[], int isperiodic_x,
                              int isperiodic_y) {
    EntryLock lk;
    AosArgs a;
    const size_t N = (size_t)Nx * Ny;
    if (!check_lattice(Q, cx, cy, opp) || !aos_begin(a, Nx, Ny, isperiodic_x, isperiodic_y))
        return report("interpolated_bounce_back");
    void *p;
    bool okk = up(SL_F, f, N * 9 * 8, &p); a.f = (double *)p;
    okk = okk && up(SL_FNEW, f_new, N * 9 * 8, &p); a.fnew = (double *)p;
    okk = okk && up(SL_MASK, solid_mask, N * 4, &p); a.mask = (int *)p;
    okk = okk && up(SL_PHI, phi, N * 8, &p); a.phi = (double *)p;
    okk = okk && check_cuda(launch::aos_op(AOS_IBB, a, g_scr.s), "ibb") &&
          down(f_new, a.fnew, N * 9 * 8) && check_cuda(cudaStreamSynchronize(g_scr.s), "ibb");
    if (!okk) report("interpolated_bounce_back");
}

}  // extern "C"

// Standalone edge BC (any of lbc's BCFunction-typed functions).
static void run_bc(const char *name, int kind, int Nx, int Ny, int Q, int index, const double *val1,
                   const double *val2, double *f, double *f_new, double *rho, double *u, double *v,
                   int *solid_mask, int cx[], int cy[], double w[]) {
    EntryLock lk;
    AosArgs a;
    const size_t N = (size_t)Nx * Ny;
    if (!check_lattice(Q, cx, cy, nullptr) || !aos_begin(a, Nx, Ny, 0, 0)) return report(name);
    const bool per = kind == BC_PERIODIC_X || kind == BC_PERIODIC_Y;
    const bool col = bc_is_column(kind);
    const int along = per ? (kind == BC_PERIODIC_X ? 2 * Ny : 2 * Nx) : (col ? Ny : Nx);
    if (!per && (index < 0 || index >= (col ? Nx : Ny))) {
        set_error("BC index out of range");
        return report(name);
    }
    void *p;
    bool okk = up(SL_FNEW, f_new, N * 9 * 8, &p); a.fnew = (double *)p;
    okk = okk && up(SL_MASK, solid_mask, N * 4, &p); a.mask = (int *)p;
    if (per) { okk = okk && up(SL_F, f, N * 9 * 8, &p); a.f = (double *)p; }
    const bool needs_fields = !per && kind != BC_VEL_IN_ZH && kind != BC_VEL_OUT_ZH &&
                              kind != BC_VEL_TOP_ZH && kind != BC_VEL_BOT_ZH && kind != BC_VEL_BOT_ZH_FIX &&
                              kind != BC_CONV_IN && kind != BC_CONV_OUT;
    if (needs_fields) {
        okk = okk && up(SL_RHO, rho, N * 8, &p); a.rho = (double *)p;
        okk = okk && up(SL_U, u, N * 8, &p); a.u = (double *)p;
        okk = okk && up(SL_V, v, N * 8, &p); a.v = (double *)p;
    }
    std::vector<double> zeros(along, 0.0);
    const double *d1 = nullptr, *d2 = nullptr;
    if (!per && kind != BC_CONV_IN && kind != BC_CONV_OUT) {
        okk = okk && up(SL_VAL1, val1 ? val1 : zeros.data(), along * 8, &p); d1 = (double *)p;
        okk = okk && up(SL_VAL2, val2 ? val2 : zeros.data(), along * 8, &p); d2 = (double *)p;
    }
    for (int k = 0; k < 9; k++) a.w[k] = w[k];
    okk = okk && check_cuda(launch::aos_bc(a, kind, index, along, d1, d2, g_scr.s), name) &&
          down(f_new, a.fnew, N * 9 * 8) && check_cuda(cudaStreamSynchronize(g_scr.s), name);
    if (!okk) report(name);
}

#define LBM_DEFINE_BC(fname, kind)                                                             \
    extern "C" void fname(int Nx, int Ny, int Q, int index, const double *val1,                \
                          const double *val2, double *f, double *f_new, double *rho, double *u, \
                          double *v, int *solid_mask, int cx[], int cy[], double w[]) {        \
        run_bc(#fname, kind, Nx, Ny, Q, index, val1, val2, f, f_new, rho, u, v, solid_mask, cx, \
               cy, w);                                                                         \
    }

// lbc src/bc/*.c, one definition each (see lbm_bc.h for the citations).
LBM_DEFINE_BC(velocity_inlet, BC_VEL_IN_ZH)
LBM_DEFINE_BC(velocity_outlet, BC_VEL_OUT_ZH)
LBM_DEFINE_BC(velocity_top, BC_VEL_TOP_ZH)
LBM_DEFINE_BC(velocity_bottom, BC_VEL_BOT_ZH)
LBM_DEFINE_BC(pressure_inlet, BC_PRES_IN_ZH)
LBM_DEFINE_BC(pressure_outlet, BC_PRES_OUT_ZH)
LBM_DEFINE_BC(convective_inlet, BC_CONV_IN)
LBM_DEFINE_BC(convective_outlet, BC_CONV_OUT)
LBM_DEFINE_BC(periodic_x, BC_PERIODIC_X)
LBM_DEFINE_BC(periodic_y, BC_PERIODIC_Y)
LBM_DEFINE_BC(velocity_inlet_regularized, BC_VEL_IN_REG)
LBM_DEFINE_BC(velocity_outlet_regularized, BC_VEL_OUT_REG)
LBM_DEFINE_BC(velocity_top_regularized, BC_VEL_TOP_REG)
LBM_DEFINE_BC(velocity_bottom_regularized, BC_VEL_BOT_REG)
LBM_DEFINE_BC(pressure_inlet_regularized, BC_PRES_IN_REG)
LBM_DEFINE_BC(pressure_outlet_regularized, BC_PRES_OUT_REG)
LBM_DEFINE_BC(pressure_top_regularized, BC_PRES_TOP_REG)
LBM_DEFINE_BC(pressure_bottom_regularized, BC_PRES_BOT_REG)
// extension: the corrected Zou-He bottom closure (lbm_bc.h)
LBM_DEFINE_BC(velocity_bottom_corrected, BC_VEL_BOT_ZH_FIX)

extern "C" {

// ------------------------------------------------------------------ Mei initialisation
// src/core/mei_initialization.c:7-143 on the GPU. The mean density is summed on
// the host in lbc's order (:42-48) so the start populations match bit for bit.
void mei_initialization(int Nx, int Ny, int Q, double *f, double *f_new, double *rho_in,
                        double *U_in, double *V_in, double *rho, double *u, double *v, int cx[],
                        int cy[], double w[], double *omega_eff, int isperiodic_x,
                        int isperiodic_y, int init_iter_max, double tol_rho, int *solid_mask) {
    EntryLock lk;
    printf("Initialization of the populations... ");
    AosArgs a;
    const size_t N = (size_t)Nx * Ny;
    if (!check_lattice(Q, cx, cy, nullptr) || !aos_begin(a, Nx, Ny, isperiodic_x, isperiodic_y))
        return report("mei_initialization");
    double rho0 = 0.0;
    for (size_t n = 0; n < N; n++) rho0 += rho_in[n];
    rho0 /= (Nx * Ny);
    void *p;
    bool okk = up(SL_F, f, N * 9 * 8, &p);  // content irrelevant, overwritten below
    double *A = (double *)p;
    okk = okk && up(SL_FNEW, f_new, N * 9 * 8, &p);
    double *B = (double *)p;
    okk = okk && up(SL_RHO, rho_in, N * 8, &p); a.rho = (double *)p;
    okk = okk && up(SL_U, U_in, N * 8, &p); a.u = (double *)p;
    okk = okk && up(SL_V, V_in, N * 8, &p); a.v = (double *)p;
    okk = okk && up(SL_OMEGA, omega_eff, N * 8, &p); a.omega = (double *)p;
    okk = okk && up(SL_MASK, solid_mask, N * 4, &p); a.mask = (int *)p;
    unsigned long long *maxbits = (unsigned long long *)g_scr.get(SL_TICK, 16);
    for (int k = 0; k < 9; k++) a.w[k] = w[k];
    if (!okk || !maxbits) return report("mei_initialization");
    a.f = A;
    if (!check_cuda(launch::mei_init(a, rho0, g_scr.s), "mei")) return report("mei_initialization");
    double maxd = 0.0;
    double *cur = A, *oth = B;
    for (int it = 0; it < init_iter_max; it++) {
        a.f = cur;
        a.fnew = oth;
        if (!check_cuda(cudaMemsetAsync(maxbits, 0, 8, g_scr.s), "mei") ||
            !check_cuda(launch::mei_iter(a, rho0, maxbits, g_scr.s), "mei") ||
            !check_cuda(launch::aos_op(AOS_STREAMING, a, g_scr.s), "mei"))
            return report("mei_initialization");
        double *t = cur; cur = oth; oth = t;
        unsigned long long bits = 0;
        if (!down(&bits, maxbits, 8) || !check_cuda(cudaStreamSynchronize(g_scr.s), "mei"))
            return report("mei_initialization");
        std::memcpy(&maxd, &bits, 8);
        if (maxd <= tol_rho) {
            printf("Initialization converged at iter %d with max |drho| = %g\n", it, maxd);
            break;
        }
    }
    if (maxd > tol_rho)
        printf("Initialization not converged after %d iterations (max |drho| = %g)\n", init_iter_max, maxd);
    okk = down(f, A, N * 9 * 8) && down(f_new, B, N * 9 * 8) && down(rho, a.rho, N * 8) &&
          check_cuda(cudaStreamSynchronize(g_scr.s), "mei");
    if (!okk) return report("mei_initialization");
    std::memcpy(u, U_in, N * 8);
    std::memcpy(v, V_in, N * 8);
}

// ------------------------------------------------------------------ host utilities

// src/core/sponge_layer.c:3-45: per-node omega = 1/tau with a radial exponential
// ramp of tau between r_inner and r_outer, filled on the device (k_sponge) and
// written to the caller's array.
void sponge_layer(int Nx, int Ny, double dx, double xc, double yc, double r_inner, double r_outer,
                  double tau_base, double incr_tau, double exp_coeff, double *omega_eff) {
    EntryLock lk;
    AosArgs a;
    const size_t N = (size_t)Nx * Ny;
    if (!omega_eff || !aos_begin(a, Nx, Ny, 0, 0)) return report("sponge_layer");
    double *d = (double *)g_scr.get(SL_OMEGA, N * 8);
    const bool okk = d &&
                     check_cuda(launch::sponge(Nx, Ny, dx, xc, yc, r_inner, r_outer, tau_base, incr_tau, exp_coeff,
                                               d, g_scr.s), "sponge_layer") &&
                     down(omega_eff, d, N * 8) && check_cuda(cudaStreamSynchronize(g_scr.s), "sponge_layer");
    if (!okk) report("sponge_layer");
}

// src/utils/filesystem.c:38-57 (POSIX branch).
int ensure_directory_exists(const char *path) {
    struct stat st;
    if (stat(path, &st) == 0) {
        if (S_ISDIR(st.st_mode)) return 0;
        fprintf(stderr, "Path exists but is not a directory: %s\n", path);
        return -1;
    }
    if (mkdir(path, 0755) != 0) {
        perror("mkdir failed");
        return -1;
    }
    return 0;
}

static inline void put_be32(unsigned char *dst, float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    dst[0] = (unsigned char)(b >> 24);
    dst[1] = (unsigned char)(b >> 16);
    dst[2] = (unsigned char)(b >> 8);
    dst[3] = (unsigned char)b;
}

// src/utils/write_vtk_binary_2D.c:25-84: legacy VTK, ASCII header, big-endian
// FP32 payload (velocity as 3-vectors with z = 0, then density).
void write_vtk_binary_2D(const char *filename, int Nx, int Ny, double dx, double *u, double *v,
                         double *rho, double cu, double crho) {
    EntryLock lk;
    FILE *fd = fopen(filename, "wb");
    if (!fd) {
        perror("Failed to open VTK file");
        return;
    }
    fprintf(fd, "# vtk DataFile Version 3.0\n2D LBM output\nBINARY\nDATASET STRUCTURED_POINTS\n");
    fprintf(fd, "DIMENSIONS %d %d 1\n", Nx, Ny);
    fprintf(fd, "ORIGIN 0 0 0\n");
    fprintf(fd, "SPACING %f %f 1\n", dx, dx);
    fprintf(fd, "\nPOINT_DATA %d\n", Nx * Ny);
    const size_t N = (size_t)Nx * Ny;
    std::vector<unsigned char> vel(N * 12), den(N * 4);
    for (size_t n = 0; n < N; n++) {
        put_be32(&vel[n * 12], (float)(u[n] * cu));
        put_be32(&vel[n * 12 + 4], (float)(v[n] * cu));
        put_be32(&vel[n * 12 + 8], 0.0f);
        put_be32(&den[n * 4], (float)(rho[n] * crho));
    }
    fprintf(fd, "VECTORS velocity float\n");
    fwrite(vel.data(), 1, vel.size(), fd);
    fprintf(fd, "\nSCALARS density float 1\n");
    fprintf(fd, "LOOKUP_TABLE default\n");
    fwrite(den.data(), 1, den.size(), fd);
    fclose(fd);
}

// ------------------------------------------------------------------ extended API

struct lbm_gpu_solver {
    std::unique_ptr<Solver> s;
};

const char *lbm_gpu_last_error(void) { return last_error(); }

int lbm_gpu_host_access(const void *p) {
    int dev = 0, pageable = 0, via_tables = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
    cudaDeviceGetAttribute(&via_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
    if (p) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, p) == cudaSuccess && a.type == cudaMemoryTypeHost &&
            a.devicePointer == p)
            return 1;
        cudaGetLastError();
    }
    return (pageable && via_tables) ? 2 : 0;
}

int lbm_gpu_fp64_rate(double *lane_ops_per_s) {
    if (!lane_ops_per_s) { set_error("null argument"); return LBM_GPU_ERR_ARG; }
    int dev = 0, sms = 0;
    if (!check_cuda(cudaGetDevice(&dev), "cudaGetDevice") ||
        !check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"))
        return LBM_GPU_ERR_CUDA;
    double *sink = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int blocks = 8 * sms, iters = 4096;
    float best = 0.f;
    bool okk = check_cuda(cudaMalloc(&sink, sizeof(double)), "cudaMalloc") &&
               check_cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate") &&
               check_cuda(cudaEventCreate(&e0), "cudaEventCreate") && check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
    // One warm-up launch, then the fastest of five.
    for (int rep = 0; okk && rep < 6; rep++) {
        float ms = 0.f;
        okk = check_cuda(cudaEventRecord(e0, s), "cudaEventRecord") &&
              check_cuda(launch::fp64_rate(blocks, iters, sink, s), "k_fp64_rate") &&
              check_cuda(cudaEventRecord(e1, s), "cudaEventRecord") &&
              check_cuda(cudaEventSynchronize(e1), "cudaEventSynchronize") &&
              check_cuda(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
        if (okk && rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (sink) cudaFree(sink);
    if (!okk || best <= 0.f) return LBM_GPU_ERR_CUDA;
    *lane_ops_per_s = (double)blocks * 256.0 * 8.0 * iters / (best * 1e-3);
    return LBM_GPU_OK;
}

int lbm_gpu_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

int lbm_gpu_create(const lbm_gpu_case *c, lbm_gpu_solver **out) {
    if (!c || !out) { set_error("null argument"); return LBM_GPU_ERR_ARG; }
    *out = nullptr;
    if (!check_lattice(9, c->cx, c->cy, c->opp)) return LBM_GPU_ERR_ARG;
    if (!c->w || !c->omega_eff) { set_error("w and omega_eff are required"); return LBM_GPU_ERR_ARG; }
    CaseDesc d;
    if (!storage_to_desc(c->storage, d)) { set_error("bad storage"); return LBM_GPU_ERR_ARG; }
    if (!fill_desc(d, c->Nx, c->Ny, c->w, c->omega_eff, c->solid_mask, c->boundaries,
                   c->num_boundaries, c->isperiodic_x, c->isperiodic_y, c->Fx, c->Fy, c->phi,
                   c->use_IBB))
        return LBM_GPU_ERR_ARG;
    d.wall_u = c->wall_u;
    d.wall_v = c->wall_v;
    std::unique_ptr<Solver> s(new Solver(d));
    if (!s->ok()) return LBM_GPU_ERR_CUDA;
    *out = new lbm_gpu_solver{std::move(s)};
    return LBM_GPU_OK;
}

int lbm_gpu_destroy(lbm_gpu_solver *s) {
    delete s;
    return LBM_GPU_OK;
}

#define SOLVER_OR_FAIL(s)                                   \
    if (!(s) || !(s)->s) {                                  \
        set_error("null solver");                           \
        return LBM_GPU_ERR_ARG;                             \
    }

int lbm_gpu_set_state(lbm_gpu_solver *s, const double *f, const double *f_new, const double *rho,
                      const double *u, const double *v) {
    SOLVER_OR_FAIL(s);
    if (!f || !f_new || !rho || !u || !v) { set_error("null array"); return LBM_GPU_ERR_ARG; }
    return s->s->set_state(f, f_new, rho, u, v) ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

int lbm_gpu_get_state(lbm_gpu_solver *s, double *f, double *f_new, double *rho, double *u,
                      double *v) {
    SOLVER_OR_FAIL(s);
    return s->s->get_state(f, f_new, rho, u, v) ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

int lbm_gpu_get_fields(lbm_gpu_solver *s, double *rho, double *u, double *v) {
    SOLVER_OR_FAIL(s);
    return s->s->get_fields(rho, u, v) ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

int lbm_gpu_set_bc_values(lbm_gpu_solver *s, int entry, const double *val1, const double *val2) {
    SOLVER_OR_FAIL(s);
    if (entry < 0 || entry >= s->s->bc_count()) {
        set_error("lbm_gpu_set_bc_values: no Boundary entry " + std::to_string(entry));
        return LBM_GPU_ERR_ARG;
    }
    return s->s->set_bc_values(entry, val1, val2) ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

int lbm_gpu_run(lbm_gpu_solver *s, int nsteps) {
    SOLVER_OR_FAIL(s);
    if (nsteps < 0) { set_error("nsteps < 0"); return LBM_GPU_ERR_ARG; }
    return s->s->run(nsteps) ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

int lbm_gpu_run_timed(lbm_gpu_solver *s, int nsteps, double *ms) {
    SOLVER_OR_FAIL(s);
    cudaEvent_t e0, e1;
    if (!check_cuda(cudaEventCreate(&e0), "event") || !check_cuda(cudaEventCreate(&e1), "event"))
        return LBM_GPU_ERR_CUDA;
    bool okk = check_cuda(cudaEventRecord(e0, s->s->stream()), "event") && s->s->run(nsteps) &&
               check_cuda(cudaEventRecord(e1, s->s->stream()), "event") &&
               check_cuda(cudaEventSynchronize(e1), "event");
    float t = 0.f;
    if (okk) okk = check_cuda(cudaEventElapsedTime(&t, e0, e1), "event");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms) *ms = t;
    return okk ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

int lbm_gpu_sync(lbm_gpu_solver *s) {
    SOLVER_OR_FAIL(s);
    if (!check_cuda(cudaStreamSynchronize(s->s->stream()), "sync")) return LBM_GPU_ERR_CUDA;
    return s->s->vtk_wait() ? LBM_GPU_OK : LBM_GPU_ERR_IO;
}

int lbm_gpu_checkpoint_save(lbm_gpu_solver *s, const char *path) {
    SOLVER_OR_FAIL(s);
    return s->s->checkpoint_save(path) ? LBM_GPU_OK : LBM_GPU_ERR_IO;
}

int lbm_gpu_checkpoint_load(lbm_gpu_solver *s, const char *path) {
    SOLVER_OR_FAIL(s);
    return s->s->checkpoint_load(path) ? LBM_GPU_OK : LBM_GPU_ERR_IO;
}

int lbm_gpu_write_vtk(lbm_gpu_solver *s, const char *filename, double dx, double cu, double crho) {
    SOLVER_OR_FAIL(s);
    return s->s->write_vtk(filename, dx, cu, crho) ? LBM_GPU_OK : LBM_GPU_ERR_IO;
}

int lbm_gpu_forces(lbm_gpu_solver *s, double *L, double *D) {
    SOLVER_OR_FAIL(s);
    return s->s->forces(D, L) ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

long long lbm_gpu_write_force_records(lbm_gpu_solver *s, const char *path, double dt, double cf, int append) {
    SOLVER_OR_FAIL(s);
    if (!path) { set_error("null path"); return LBM_GPU_ERR_ARG; }
    const long long n = s->s->write_force_records(path, dt, cf, append != 0);
    return n >= 0 ? n : (n == -2 ? LBM_GPU_ERR_ARG : LBM_GPU_ERR_IO);
}

int lbm_gpu_set_probes(lbm_gpu_solver *s, int n, const int *i, const int *j, int capacity) {
    SOLVER_OR_FAIL(s);
    return s->s->set_probes(n, i, j, capacity) ? LBM_GPU_OK : LBM_GPU_ERR_ARG;
}

int lbm_gpu_probe_history(lbm_gpu_solver *s, double *out, int max_steps) {
    SOLVER_OR_FAIL(s);
    if (!out || max_steps < 0) { set_error("bad arguments"); return LBM_GPU_ERR_ARG; }
    const int n = s->s->probe_history(out, max_steps);
    return n < 0 ? LBM_GPU_ERR_CUDA : n;
}

int lbm_gpu_enable_impedance_trace(lbm_gpu_solver *s, int entry, int capacity) {
    SOLVER_OR_FAIL(s);
    return s->s->enable_impedance_trace(entry, capacity) ? LBM_GPU_OK : LBM_GPU_ERR_ARG;
}

long long lbm_gpu_write_impedance_trace(lbm_gpu_solver *s, int entry, const char *path, double dt, double cp,
                                        double cu, int append) {
    SOLVER_OR_FAIL(s);
    if (!path) { set_error("null path"); return LBM_GPU_ERR_ARG; }
    const long long n = s->s->write_impedance_trace(entry, path, dt, cp, cu, append != 0);
    if (n == -2) return LBM_GPU_ERR_ARG;
    return n < 0 ? LBM_GPU_ERR_IO : n;
}

int lbm_gpu_enable_force_history(lbm_gpu_solver *s, int capacity) {
    SOLVER_OR_FAIL(s);
    return s->s->enable_force_history(capacity) ? LBM_GPU_OK : LBM_GPU_ERR_ARG;
}

int lbm_gpu_force_history(lbm_gpu_solver *s, double *xy, int max_steps) {
    SOLVER_OR_FAIL(s);
    return s->s->force_history(xy, max_steps);
}

int lbm_gpu_set_impedance_wall(lbm_gpu_solver *s, int entry, const double *R, const double *m,
                               const double *K, int nf, const double *omegas, double rho_ref,
                               double alpha, int window_steps) {
    SOLVER_OR_FAIL(s);
    if (!R || !m || !K || (nf > 0 && !omegas)) { set_error("null array"); return LBM_GPU_ERR_ARG; }
    return s->s->set_impedance(entry, R, m, K, nf, omegas, rho_ref, alpha, window_steps) ? LBM_GPU_OK
                                                                                        : LBM_GPU_ERR_ARG;
}

int lbm_gpu_impedance_readback(lbm_gpu_solver *s, int entry, double *spectra, double *state) {
    SOLVER_OR_FAIL(s);
    return s->s->impedance_readback(entry, spectra, state) ? LBM_GPU_OK : LBM_GPU_ERR_ARG;
}

int lbm_gpu_msd_zoh(double R, double m, double K, double *A, double *b) {
    if (!A || !b) { set_error("null array"); return LBM_GPU_ERR_ARG; }
    if (!msd_zoh(R, m, K, A, b)) { set_error("need m > 0, K > 0, R >= 0"); return LBM_GPU_ERR_ARG; }
    return LBM_GPU_OK;
}

int lbm_gpu_get_info(lbm_gpu_solver *s, lbm_gpu_info *info) {
    SOLVER_OR_FAIL(s);
    info->Nx = s->s->Nx();
    info->Ny = s->s->Ny();
    info->pitch = s->s->pitch();
    info->storage = s->s->storage_code();
    info->has_geometry = s->s->has_flags() ? 1 : 0;
    info->edge_stages = s->s->nstages();
    info->launches_per_step = s->s->launches_per_step();
    info->edge_launches = (int)s->s->stage_groups().size();
    info->device_bytes = s->s->device_bytes();
    info->steps_done = s->s->steps_done();
    return LBM_GPU_OK;
}

int lbm_gpu_set_block(lbm_gpu_solver *s, int bx, int by) {
    SOLVER_OR_FAIL(s);
    if (bx < 32 || by < 1 || bx % 32 != 0 || bx * by > 256) {
        set_error("block must be bx*by <= 256 with bx a multiple of 32");
        return LBM_GPU_ERR_ARG;
    }
    return s->s->set_block(dim3(bx, by, 1)) ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

int lbm_gpu_get_block(lbm_gpu_solver *s, int *bx, int *by) {
    SOLVER_OR_FAIL(s);
    if (bx) *bx = (int)s->s->block().x;
    if (by) *by = (int)s->s->block().y;
    return LBM_GPU_OK;
}

int lbm_gpu_set_autotune(lbm_gpu_solver *s, int mode) {
    SOLVER_OR_FAIL(s);
    s->s->set_autotune(mode);
    return LBM_GPU_OK;
}

int lbm_gpu_autotune_status(lbm_gpu_solver *s, int *tuned, int *bx, int *by, double *us_per_step) {
    SOLVER_OR_FAIL(s);
    if (tuned) *tuned = s->s->tuned() ? 1 : 0;
    if (bx) *bx = (int)s->s->block().x;
    if (by) *by = (int)s->s->block().y;
    if (us_per_step) *us_per_step = s->s->tuned_us();
    return LBM_GPU_OK;
}

void lbm_gpu_tune_cache_clear(void) { tune_clear(); }

struct lbm_gpu_batch {
    std::unique_ptr<Batch> b;
};

int lbm_gpu_batch_create(lbm_gpu_solver *const *solvers, int n, lbm_gpu_batch **out) {
    if (!solvers || n <= 0 || !out) { set_error("bad arguments"); return LBM_GPU_ERR_ARG; }
    *out = nullptr;
    std::vector<Solver *> v;
    for (int i = 0; i < n; i++) {
        if (!solvers[i] || !solvers[i]->s) { set_error("null solver in batch"); return LBM_GPU_ERR_ARG; }
        v.push_back(solvers[i]->s.get());
    }
    std::unique_ptr<Batch> b(new Batch(v));
    if (!b->ok()) return LBM_GPU_ERR_CUDA;
    *out = new lbm_gpu_batch{std::move(b)};
    return LBM_GPU_OK;
}

int lbm_gpu_batch_run(lbm_gpu_batch *b, int nsteps) {
    if (!b || nsteps < 0) { set_error("bad arguments"); return LBM_GPU_ERR_ARG; }
    return b->b->run(nsteps) ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

int lbm_gpu_batch_run_timed(lbm_gpu_batch *b, int nsteps, double *ms) {
    if (!b || nsteps < 0) { set_error("bad arguments"); return LBM_GPU_ERR_ARG; }
    cudaEvent_t e0, e1;
    if (!check_cuda(cudaEventCreate(&e0), "event") || !check_cuda(cudaEventCreate(&e1), "event"))
        return LBM_GPU_ERR_CUDA;
    bool okk = check_cuda(cudaEventRecord(e0, b->b->stream()), "event") && b->b->run(nsteps) &&
               check_cuda(cudaEventRecord(e1, b->b->stream()), "event") &&
               check_cuda(cudaEventSynchronize(e1), "event");
    float t = 0.f;
    if (okk) okk = check_cuda(cudaEventElapsedTime(&t, e0, e1), "event");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms) *ms = t;
    return okk ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

int lbm_gpu_batch_info(lbm_gpu_batch *b, long long *nodes, int *launches_per_step) {
    if (!b) { set_error("null batch"); return LBM_GPU_ERR_ARG; }
    if (nodes) *nodes = b->b->nodes();
    if (launches_per_step) *launches_per_step = b->b->launches_per_step();
    return LBM_GPU_OK;
}

int lbm_gpu_batch_set_tile(lbm_gpu_batch *b, int tw, int th) {
    if (!b) { set_error("null batch"); return LBM_GPU_ERR_ARG; }
    int tws = -1;
    for (int q = 5; q <= 8; q++)
        if (tw == (1 << q) && th == (256 >> q)) tws = q;
    if (tws < 0) {
        set_error("batch tile must be tw x th = 256 with tw in {32, 64, 128, 256}");
        return LBM_GPU_ERR_ARG;
    }
    return b->b->set_tile_shift(tws) ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

int lbm_gpu_batch_set_autotune(lbm_gpu_batch *b, int mode) {
    if (!b) { set_error("null batch"); return LBM_GPU_ERR_ARG; }
    b->b->set_autotune(mode);
    return LBM_GPU_OK;
}

int lbm_gpu_batch_autotune_status(lbm_gpu_batch *b, int *tuned, int *tw, int *th, double *us_per_step) {
    if (!b) { set_error("null batch"); return LBM_GPU_ERR_ARG; }
    const int tws = b->b->tile_shift();
    if (tuned) *tuned = b->b->tuned() ? 1 : 0;
    if (tw) *tw = 1 << tws;
    if (th) *th = 256 >> tws;
    if (us_per_step) *us_per_step = b->b->tuned_us();
    return LBM_GPU_OK;
}

int lbm_gpu_batch_destroy(lbm_gpu_batch *b) {
    delete b;
    return LBM_GPU_OK;
}

void *lbm_gpu_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (!check_cuda(cudaHostAlloc(&p, bytes, cudaHostAllocDefault), "cudaHostAlloc")) return nullptr;
    return p;
}

void lbm_gpu_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

void lbm_gpu_dropin_set_staged(int staged) {
    EntryLock lk;
    g_force_staged = staged != 0;
}

void lbm_gpu_dropin_release(void) {
    EntryLock lk;
    g_cache.clear();
}

void lbm_gpu_dropin_set_lazy(int lazy) {
    EntryLock lk;
    g_lazy = lazy != 0;
}

int lbm_gpu_dropin_sync(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    return flush_lazy() ? LBM_GPU_OK : LBM_GPU_ERR_CUDA;
}

}  // extern "C"
