// engine.cpp -- host side of the GB300 D2Q9 engine.
//
// A Solver owns one case on the device:
//   * two population buffers (SoA planes, FP64 or shifted FP32/FP16), swapped
//     every step like lbc's caller swaps f/f_new (cases/nit/nit.c:309-311);
//   * a per-node flag word and a cut-link table built once from the geometry;
//   * the edge-BC band: pre-collision populations and previous-step moments of
//     the nodes lbc's Boundary list writes or reads;
//   * stored macroscopic fields rho/u/v (dense [Ny][Nx], FP64).
// Solver::run(n) is equivalent to n calls of lbc's main_lbm plus the caller-side
// swap: it collides the current state with the stored fields (as lbc's first
// call does), runs n-1 fused steps from a two-step CUDA graph, and ends with a
// step that stores pre-collision populations and the moments, so the state at
// exit is what lbc's arrays hold after n calls.
#include "engine.h"
#include "tune.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <unordered_set>

namespace lbm {

static thread_local std::string g_err;

void set_error(const std::string &msg) { g_err = msg; }
const char *last_error() { return g_err.c_str(); }

bool check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

#define CK(call)                                \
    do {                                        \
        if (!check_cuda((call), #call)) return false; \
    } while (0)

// Device memory is stream-ordered (cudaMallocAsync / cudaFreeAsync on the
// owner's stream, from the device's default pool): freeing a finished case
// does not synchronize the device, so a server can retire cases while other
// batches run.
void use_retaining_pool() {
    static std::mutex mu;
    static std::set<int> done;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    std::lock_guard<std::mutex> lk(mu);
    if (done.count(dev)) return;
    done.insert(dev);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) return;
    unsigned long long keep = ~0ull;  // keep freed blocks for reuse instead of returning them
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
}

bool device_alloc(void **q, size_t bytes, cudaStream_t s) {
    return check_cuda(cudaMallocAsync(q, bytes, s), "cudaMallocAsync");
}

template <class T> bool Solver::dalloc(T **p, size_t count) {
    if (count == 0) count = 1;
    void *q = nullptr;
    if (!device_alloc(&q, count * sizeof(T), stream_)) return false;
    allocs_.push_back(q);
    dev_bytes_ += count * sizeof(T);
    *p = (T *)q;
    return true;
}

Solver::Solver(const CaseDesc &d) : d_(d) {
    if (d_.Nx < 2 || d_.Ny < 2) {
        set_error("grid must be at least 2 x 2");
        return;
    }
    if (d_.fma64) {
        const double *w = d_.w;
        if (d_.store != STORE_F64 || !(w[1] == w[2] && w[1] == w[3] && w[1] == w[4] && w[5] == w[6] &&
                                       w[5] == w[7] && w[5] == w[8])) {
            set_error("FP64 FMA storage needs FP64 storage and lbc's weight symmetry (w1..w4 equal, w5..w8 equal)");
            return;
        }
    }
    esize_ = d_.store == STORE_F64 ? 8 : (d_.store == STORE_F32 ? 4 : 2);
    pitch_ = (d_.Nx + 63) / 64 * 64;
    plane_ = (long long)pitch_ * d_.Ny;
    // Highest stream priority: a case's own work is short (setup, a run
    // alone, results), and when a server admits it while batches run, its
    // setup kernels take the next free SMs instead of waiting for a gap
    // between the batches' steps.
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (!check_cuda(cudaStreamCreateWithPriority(&stream_, cudaStreamNonBlocking, hi), "cudaStreamCreate")) return;
    use_retaining_pool();
    if (!build_geometry()) return;
    ok_ = true;
    set_autotune(tune_default_mode());
}

Solver::~Solver() {
    vtk_wait();
    if (vtk_ev_) cudaEventDestroy(vtk_ev_);
    if (h_vtk_) cudaFreeHost(h_vtk_);
    if (pair_exec_) cudaGraphExecDestroy(pair_exec_);
    for (void *p : allocs_) cudaFreeAsync(p, stream_);
    if (stream_) cudaStreamDestroy(stream_);
}

static inline bool wrap(int &c, int n, int periodic) {
    if (periodic) {
        if (c < 0) c += n;
        else if (c >= n) c -= n;
        return true;
    }
    return c >= 0 && c < n;
}

// Geometry preprocessing (once per case):
//   flags: solid bit; bit k when the pull source x - c_k is solid or off a
//          non-periodic edge; band/BC-write bits; link bit.
//   links: per fluid node with solid sources, one entry per such source in k
//          order: interpolated bounce-back coefficients computed exactly as
//          src/bc/interpolated_bounce_back.c:52-99 does, or the moving-wall term.
//   band:  the columns/rows lbc's Boundary list writes or reads.
bool Solver::build_geometry() {
    const int Nx = d_.Nx, Ny = d_.Ny;
    const size_t N = (size_t)Nx * Ny;
    auto solid = [&](int i, int j) { return d_.mask && d_.mask[(size_t)j * Nx + i] != 0; };

    // Uniform omega becomes a scalar.
    bool uniform = true;
    omega0_ = d_.omega ? d_.omega[0] : 1.0;
    if (d_.omega)
        for (size_t n = 1; n < N && uniform; n++) uniform = (d_.omega[n] == omega0_);

    // Stages from the Boundary list.
    bool nonperiodic_seen = false;
    for (size_t e = 0; e < d_.bcs.size(); e++) {
        const BCEntry &b = d_.bcs[e];
        if (b.kind < 0 || b.kind >= BC_KIND_COUNT) {
            set_error("boundary entry " + std::to_string(e) + ": unknown BC function");
            return false;
        }
        const bool per = b.kind == BC_PERIODIC_X || b.kind == BC_PERIODIC_Y;
        if (per) {
            // A periodic entry re-copies what the wrap in streaming already wrote
            // (src/bc/periodic_x.c vs src/core/streaming.c:24-34); it only matters
            // when its flag is off or an earlier entry overwrote the edge.
            const int flag = b.kind == BC_PERIODIC_X ? d_.px : d_.py;
            if (flag && !nonperiodic_seen) continue;
            Stage st{b.kind, 0, b.kind == BC_PERIODIC_X ? 2 * Ny : 2 * Nx, (int)e, {}};
            st.open.assign(st.along, 1);
            stages_.push_back(st);
            continue;
        }
        nonperiodic_seen = true;
        const bool col = bc_is_column(b.kind);
        const int lim = col ? Nx : Ny;
        if (b.index < 0 || b.index >= lim) {
            set_error("boundary entry " + std::to_string(e) + ": index out of range");
            return false;
        }
        Stage st{b.kind, b.index, col ? Ny : Nx, (int)e, {}};
        st.open.resize(st.along);
        for (int t = 0; t < st.along; t++) st.open[t] = col ? !solid(b.index, t) : !solid(t, b.index);
        stages_.push_back(st);
    }

    // Band lines.
    std::set<int> cols, rows, wcols, wrows;
    for (const Stage &st : stages_) {
        const int k = st.kind, x = st.index;
        auto need = [&](bool col, int idx, bool write) -> bool {
            const int lim = col ? Nx : Ny;
            if (idx < 0 || idx >= lim) {
                set_error("boundary entry " + std::to_string(st.entry) +
                          ": the BC reads a line outside the grid");
                return false;
            }
            (col ? cols : rows).insert(idx);
            if (write) (col ? wcols : wrows).insert(idx);
            return true;
        };
        bool okk = true;
        switch (k) {
        case BC_PERIODIC_X: okk = need(true, 0, true) && need(true, Nx - 1, true); break;
        case BC_PERIODIC_Y: okk = need(false, 0, true) && need(false, Ny - 1, true); break;
        case BC_VEL_IN_ZH: case BC_VEL_OUT_ZH: okk = need(true, x, true); break;
        case BC_VEL_TOP_ZH: case BC_VEL_BOT_ZH: case BC_VEL_BOT_ZH_FIX: okk = need(false, x, true); break;
        case BC_PRES_IN_ZH: case BC_CONV_IN: case BC_VEL_IN_REG: case BC_PRES_IN_REG:
            okk = need(true, x, true) && need(true, x + 1, false); break;
        case BC_PRES_OUT_ZH: case BC_CONV_OUT: case BC_VEL_OUT_REG: case BC_PRES_OUT_REG:
            okk = need(true, x, true) && need(true, x - 1, false); break;
        case BC_VEL_BOT_REG: case BC_PRES_BOT_REG: okk = need(false, x, true) && need(false, x + 1, false); break;
        case BC_VEL_TOP_REG: case BC_PRES_TOP_REG: okk = need(false, x, true) && need(false, x - 1, false); break;
        default: break;
        }
        if (!okk) return false;
    }
    std::vector<int> colbase(Nx, -1), rowbase(Ny, -1);
    int ns = 0;
    for (int c : cols) { colbase[c] = ns; ns += Ny; }
    for (int r : rows) { rowbase[r] = ns; ns += Nx; }
    nslots_ = ns;
    if (!group_stages(solid, colbase, rowbase)) return false;
    auto slot_of = [&](int i, int j) { return colbase[i] >= 0 ? colbase[i] + j : rowbase[j] + i; };

    // Flags and links.
    std::vector<uint16_t> flags((size_t)pitch_ * Ny, 0);
    std::vector<int> link_off;
    std::vector<Link> links;
    const bool moving = d_.wall_u || d_.wall_v;
    if (moving && d_.use_ibb) {
        set_error("moving walls and interpolated bounce-back cannot be combined");
        return false;
    }
    const bool want_links = d_.use_ibb || moving;
    if (want_links) link_off.assign((size_t)pitch_ * Ny, 0);
    link_node_.assign((size_t)Nx * Ny, 0);
    bool any_special = false, any_solid_link = false;
    std::vector<int2> seed_nodes;
    std::vector<int> seed_slots;
    for (int j = 0; j < Ny; j++) {
        for (int i = 0; i < Nx; i++) {
            uint16_t fl = 0;
            const size_t node = (size_t)j * pitch_ + i;
            const bool band = (colbase[i] >= 0) || (rowbase[j] >= 0);
            const bool bcw = !solid(i, j) && (wcols.count(i) || wrows.count(j));
            if (band) {
                fl |= NF_BAND;
                seed_nodes.push_back(make_int2(i, j));
                seed_slots.push_back(slot_of(i, j));
            }
            if (solid(i, j)) {
                fl |= NF_SOLID;
                flags[node] = fl;
                any_special = true;
                continue;
            }
            if (bcw) fl |= NF_BCW;
            int first_link = (int)links.size();
            bool has_link = false;
            for (int k = 1; k < 9; k++) {
                int si = i - cxk(k), sj = j - cyk(k);
                if (!wrap(si, Nx, d_.px) || !wrap(sj, Ny, d_.py)) {
                    fl |= (uint16_t)(1u << k);
                    any_special = true;
                    continue;
                }
                if (!solid(si, sj)) continue;
                fl |= (uint16_t)(1u << k);
                any_special = true;
                any_solid_link = true;
                link_node_[(size_t)j * Nx + i] = 1;
                if (!want_links) continue;
                Link L;
                std::memset(&L, 0, sizeof L);
                L.mode = LINK_BB;
                L.k = (uint8_t)k;
                L.behind = -1;
                const int kl = oppk(k);  // link direction, from x towards the solid node
                if (d_.use_ibb) {
                    const double eps = 1e-12;
                    const double phx = d_.phi[(size_t)j * Nx + i];
                    double denom = phx - d_.phi[(size_t)sj * Nx + si];
                    if (std::fabs(denom) < eps) denom = (denom >= 0.0) ? eps : -eps;
                    double q = phx / denom;
                    if (q < eps) q = eps;
                    if (q > 1.0 - eps) q = 1.0 - eps;
                    int bi = i - cxk(kl), bj = j - cyk(kl);
                    if (wrap(bi, Nx, d_.px) && wrap(bj, Ny, d_.py)) {
                        if (q <= 0.5) {
                            L.mode = LINK_IBB_LO;
                            L.c1 = 1.0 - 2.0 * q;
                            L.c2 = 2.0 * q;
                            L.behind = (int64_t)bj * pitch_ + bi;
                        } else if (!solid(bi, bj)) {
                            L.mode = LINK_IBB_HI;
                            L.c1 = 1.0 / (2.0 * q);
                            L.c2 = (2.0 * q - 1.0) / (2.0 * q);
                            L.behind = (int64_t)bj * pitch_ + bi;
                        }
                    }
                } else {
                    const size_t s = (size_t)sj * Nx + si;
                    const double uw = d_.wall_u ? d_.wall_u[s] : 0.0;
                    const double vw = d_.wall_v ? d_.wall_v[s] : 0.0;
                    const double cuw = cxk(kl) * uw + cyk(kl) * vw;
                    if (cuw != 0.0) {
                        L.mode = LINK_MOVING;
                        L.c2 = 6.0 * d_.w[kl] * cuw;
                    }
                }
                links.push_back(L);
                has_link = true;
            }
            if (has_link) {
                fl |= NF_LINKS;
                link_off[node] = first_link;
            }
            flags[node] = fl;
        }
    }
    has_flags_ = any_special || !stages_.empty() || !d_.px || !d_.py;
    // Shifted storage: the nodes the clean-pair kernels leave out (both nodes
    // of every pair (2m, 2m + 1) of a row with a special node, and the last
    // column of an odd-width grid), in row-major order. Solid nodes whose band
    // values no BC reads (off the band, or on it but the neighbour of no fluid
    // BC node: a BC reads only its node and that neighbour) are marked
    // (kSpecialSolid in x): their step only writes NaN moments on steps that
    // write the fields, with no load but the entry.
    special_host_.clear();
    if (d_.store != STORE_F64) {
        const uint16_t slow = NF_SPECIAL_MASK | NF_SOLID | NF_BAND | NF_BCW | NF_LINKS;
        std::vector<uint8_t> read_solid((size_t)std::max(nslots_, 1), 0);
        for (const Stage &st : stages_) {
            if (st.kind == BC_PERIODIC_X || st.kind == BC_PERIODIC_Y) continue;
            const bool col = bc_is_column(st.kind);
            for (int t = 0; t < st.along; t++) {
                const int i = col ? st.index : t, j = col ? t : st.index;
                if (solid(i, j)) continue;
                const int2 nb = stage_neighbour(st.kind, make_int2(i, j));  // the node's own stage thread reads
                const int ni = nb.x, nj = nb.y;
                if (ni < 0 || ni >= Nx || nj < 0 || nj >= Ny || !solid(ni, nj)) continue;
                read_solid[(size_t)slot_of(ni, nj)] = 1;
            }
        }
        auto entry = [&](int i, int j) {
            const uint16_t f = flags[(size_t)j * pitch_ + i];
            const bool unread = !(f & NF_BAND) || !read_solid[(size_t)slot_of(i, j)];
            const bool mark = (f & NF_SOLID) && unread && Nx <= kSpecialSolid;
            return make_int2(mark ? (i | kSpecialSolid) : i, j);
        };
        for (int j = 0; j < Ny; j++)
            for (int i0 = 0; i0 < Nx; i0 += 2) {
                const bool two = i0 + 1 < Nx;
                const size_t n0 = (size_t)j * pitch_ + i0;
                const bool sp = !two || (flags[n0] & slow) || (flags[n0 + 1] & slow);
                if (!sp) continue;
                special_host_.push_back(entry(i0, j));
                if (two) special_host_.push_back(entry(i0 + 1, j));
            }
    }
    nspecial_ = (int)special_host_.size();
    needs_old_dst_ = any_special;  // solid nodes or off-grid pull sources
    has_links_ = want_links && !links.empty();
    has_mem_ = any_solid_link;
    nseed_ = (int)seed_nodes.size();

    // Device allocation.
    for (int b = 0; b < 2; b++) {
        void *p = nullptr;
        if (!device_alloc(&p, (size_t)plane_ * 9 * esize_, stream_)) return false;
        allocs_.push_back(p);
        dev_bytes_ += (size_t)plane_ * 9 * esize_;
        buf_[b] = p;
        CK(cudaMemsetAsync(p, 0, (size_t)plane_ * 9 * esize_, stream_));
    }
    if (!dalloc(&d_rho_, N) || !dalloc(&d_ux_, N) || !dalloc(&d_uy_, N)) return false;
    stage_rows_ = staging_rows(Nx, Ny);
    if (!dalloc(&d_stage_, (size_t)stage_rows_ * Nx * 9)) return false;
    if (has_flags_) {
        if (!dalloc(&d_flags_, flags.size())) return false;
        CK(cudaMemcpyAsync(d_flags_, flags.data(), flags.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, stream_));
    }
    if (has_flags_) {
        // Clean 64-node row segments (every pair (2m, 2m + 1) in it exists and
        // is not special): the geometry kernels skip their flag words.
        const uint16_t slow = NF_SPECIAL_MASK | NF_SOLID | NF_BAND | NF_BCW | NF_LINKS;
        const int nseg = (Nx + 63) / 64;
        seg_words_ = (nseg + 31) / 32;
        std::vector<uint32_t> bits((size_t)seg_words_ * Ny, 0);
        for (int j = 0; j < Ny; j++)
            for (int sg = 0; sg < nseg; sg++) {
                bool clean = 64 * sg + 64 <= Nx;
                for (int i = 64 * sg; clean && i < 64 * sg + 64; i++) clean = !(flags[(size_t)j * pitch_ + i] & slow);
                if (clean) bits[(size_t)j * seg_words_ + sg / 32] |= 1u << (sg % 32);
            }
        if (!dalloc(&d_seg_clean_, bits.size())) return false;
        CK(cudaMemcpyAsync(d_seg_clean_, bits.data(), bits.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, stream_));
    }
    if (nspecial_) {
        if (!dalloc(&d_special_, special_host_.size())) return false;
        CK(cudaMemcpyAsync(d_special_, special_host_.data(), special_host_.size() * sizeof(int2), cudaMemcpyHostToDevice, stream_));
    }
    if (has_links_) {
        if (!dalloc(&d_link_off_, link_off.size()) || !dalloc(&d_links_, links.size())) return false;
        CK(cudaMemcpyAsync(d_link_off_, link_off.data(), link_off.size() * sizeof(int), cudaMemcpyHostToDevice, stream_));
        CK(cudaMemcpyAsync(d_links_, links.data(), links.size() * sizeof(Link), cudaMemcpyHostToDevice, stream_));
    }
    if (!uniform) {
        if (!dalloc(&d_omega_, N)) return false;
        CK(cudaMemcpyAsync(d_omega_, d_.omega, N * sizeof(double), cudaMemcpyHostToDevice, stream_));
    }
    if (nslots_ > 0) {
        if (!dalloc(&d_colbase_, (size_t)Nx) || !dalloc(&d_rowbase_, (size_t)Ny)) return false;
        CK(cudaMemcpyAsync(d_colbase_, colbase.data(), Nx * sizeof(int), cudaMemcpyHostToDevice, stream_));
        CK(cudaMemcpyAsync(d_rowbase_, rowbase.data(), Ny * sizeof(int), cudaMemcpyHostToDevice, stream_));
        // Band populations: FP64 f for FP64 storage, FP32 g = f - w otherwise.
        const bool band_ok = d_.store == STORE_F64 ? dalloc(&d_bandf_, (size_t)nslots_ * 9)
                                                   : dalloc(&d_bandg_, (size_t)nslots_ * 9);
        if (!band_ok || !dalloc(&d_bandm_[0], (size_t)nslots_ * 3) ||
            !dalloc(&d_bandm_[1], (size_t)nslots_ * 3))
            return false;
        if (!dalloc(&d_seed_nodes_, seed_nodes.size()) ||
            !dalloc(&d_seed_slots_, seed_slots.size()))
            return false;
        if (!dalloc(&d_last_, last_host_.size())) return false;
        CK(cudaMemcpyAsync(d_last_, last_host_.data(), last_host_.size() * sizeof(short), cudaMemcpyHostToDevice, stream_));
        if (nseed_) {
            CK(cudaMemcpyAsync(d_seed_nodes_, seed_nodes.data(), seed_nodes.size() * sizeof(int2), cudaMemcpyHostToDevice, stream_));
            CK(cudaMemcpyAsync(d_seed_slots_, seed_slots.data(), seed_slots.size() * sizeof(int), cudaMemcpyHostToDevice, stream_));
        }
    }
    for (Stage &st : stages_) {
        if (st.kind == BC_PERIODIC_X || st.kind == BC_PERIODIC_Y) continue;
        if (!dalloc(&st.d_val1, (size_t)st.along) || !dalloc(&st.d_val2, (size_t)st.along)) return false;
        CK(cudaMemsetAsync(st.d_val1, 0, st.along * sizeof(double), stream_));
        CK(cudaMemsetAsync(st.d_val2, 0, st.along * sizeof(double), stream_));
    }
    if (has_mem_) {
        if (!dalloc(&d_mem_out_, 2) || !dalloc(&d_force_slot_, 1)) return false;
        CK(cudaMemsetAsync(d_mem_out_, 0, 2 * sizeof(double), stream_));
        if (!compute_segment_slots()) return false;
    }
    if (!upload_all_bc_values()) return false;
    CK(cudaStreamSynchronize(stream_));
    return true;
}

// Consecutive Boundary entries that touch disjoint band nodes run in one
// launch. Entry s joins the current group unless it writes a node the group
// reads or writes, or reads a node the group writes (lbc applies the list in
// order, so such an entry must see, or must not yet see, the earlier writes).
// Writes: the entry's non-solid line nodes. Reads within the step: those nodes
// and, for entries that read their interior neighbour's populations
// (regularized, convective), the neighbour of each; moments of the previous
// step and post-collision sources (periodic entries) are not written by any
// entry.
// The last entry that writes a node also finishes it (moments, collision,
// store into the destination buffer and the band moments of the next step) in
// its own launch: no entry reads what the finish writes, and no later entry
// writes the node again. That needs one thread per node within an entry,
// which holds on every grid of at least 2 x 2 (a periodic entry on a grid one
// node wide would visit its nodes twice).
template <class Solid>
bool Solver::group_stages(const Solid &solid, const std::vector<int> &colbase, const std::vector<int> &rowbase) {
    const int Nx = d_.Nx, Ny = d_.Ny;
    groups_.clear();
    last_host_.assign((size_t)nslots_, (short)-1);
    if (stages_.size() >= 32767) {
        set_error("too many Boundary entries");
        return false;
    }
    std::unordered_set<long long> gw, gr;
    auto id = [&](int i, int j) { return (long long)j * Nx + i; };
    for (size_t s = 0; s < stages_.size(); s++) {
        const Stage &st = stages_[s];
        std::vector<long long> w, r;
        auto line = [&](bool col, int idx, int di, int dj, bool reads_neighbour) {
            const int n = col ? Ny : Nx;
            for (int t = 0; t < n; t++) {
                const int i = col ? idx : t, j = col ? t : idx;
                if (solid(i, j)) continue;
                w.push_back(id(i, j));
                r.push_back(id(i, j));
                if (reads_neighbour) r.push_back(id(i + di, j + dj));
            }
        };
        const int x = st.index;
        switch (st.kind) {
        case BC_PERIODIC_X: line(true, 0, 0, 0, false); line(true, Nx - 1, 0, 0, false); r.clear(); break;
        case BC_PERIODIC_Y: line(false, 0, 0, 0, false); line(false, Ny - 1, 0, 0, false); r.clear(); break;
        case BC_VEL_IN_ZH: case BC_VEL_OUT_ZH: case BC_PRES_IN_ZH: case BC_PRES_OUT_ZH: line(true, x, 0, 0, false); break;
        case BC_VEL_TOP_ZH: case BC_VEL_BOT_ZH: case BC_VEL_BOT_ZH_FIX: line(false, x, 0, 0, false); break;
        case BC_CONV_IN: case BC_VEL_IN_REG: case BC_PRES_IN_REG: line(true, x, 1, 0, true); break;
        case BC_CONV_OUT: case BC_VEL_OUT_REG: case BC_PRES_OUT_REG: line(true, x, -1, 0, true); break;
        case BC_VEL_BOT_REG: case BC_PRES_BOT_REG: line(false, x, 0, 1, true); break;
        case BC_VEL_TOP_REG: case BC_PRES_TOP_REG: line(false, x, 0, -1, true); break;
        default: break;
        }
        for (long long v : w) {
            const int i = (int)(v % Nx), j = (int)(v / Nx);
            const int slot = colbase[i] >= 0 ? colbase[i] + j : rowbase[j] + i;
            if (last_host_[slot] == (short)s) {
                set_error("boundary entry " + std::to_string(st.entry) + " writes a node twice");
                return false;
            }
            last_host_[slot] = (short)s;
        }
        bool conflict = groups_.empty();
        for (long long v : w)
            if (conflict || gw.count(v) || gr.count(v)) { conflict = true; break; }
        if (!conflict)
            for (long long v : r)
                if (gw.count(v)) { conflict = true; break; }
        if (conflict || groups_.back().size() >= (size_t)kStageGroupMax) {
            groups_.emplace_back();
            gw.clear();
            gr.clear();
        }
        groups_.back().push_back((int)s);
        gw.insert(w.begin(), w.end());
        gr.insert(r.begin(), r.end());
    }
    return true;
}

// Which 32-node row segments (j, i / 32) contain wall links: the warp that
// steps such a segment stores its force sum at a slot, numbered in row-major
// order. The table does not depend on the launch shape.
bool Solver::compute_segment_slots() {
    const int Nx = d_.Nx, Ny = d_.Ny;
    std::vector<int> slot;
    int n = 0;
    if (d_.store == STORE_F64) {
        // per 32-node row segment
        const int nseg = (Nx + 31) / 32;
        slot.assign((size_t)nseg * Ny, -1);
        for (int j = 0; j < Ny; j++)
            for (int g = 0; g < nseg; g++) {
                bool any = false;
                for (int i = 32 * g; i < std::min(Nx, 32 * g + 32); i++)
                    if (link_node_[(size_t)j * Nx + i]) { any = true; break; }
                if (any) slot[(size_t)j * nseg + g] = n++;
            }
    } else {
        // per 32-entry chunk of the special-node list (wall-link nodes are special)
        const int nch = (nspecial_ + 31) / 32;
        slot.assign((size_t)std::max(nch, 1), -1);
        for (int c = 0; c < nch; c++) {
            bool any = false;
            for (int q = 32 * c; q < std::min(nspecial_, 32 * c + 32); q++) {
                const int2 ij = special_host_[q];
                if (link_node_[(size_t)ij.y * Nx + (ij.x & ~kSpecialSolid)]) { any = true; break; }
            }
            if (any) slot[c] = n++;
        }
    }
    nlink_segs_ = n;
    if (!dalloc(&d_seg_slot_, slot.size()) || !dalloc(&d_partials_, 2 * (size_t)std::max(n, 1))) return false;
    CK(cudaMemcpyAsync(d_seg_slot_, slot.data(), slot.size() * sizeof(int), cudaMemcpyHostToDevice, stream_));
    CK(cudaMemsetAsync(d_partials_, 0, 2 * (size_t)std::max(n, 1) * sizeof(double), stream_));
    return upload_force_slot();
}

ForceSlot Solver::force_slot() const {
    ForceSlot f;
    std::memset(&f, 0, sizeof f);
    f.t0 = 0;
    f.t1 = nlink_segs_;
    f.partials = d_partials_;
    f.out = d_mem_out_;
    f.hist = d_hist_;
    f.hist_count = hist_count_ptr_;
    f.hist_cap = hist_cap_;
    return f;
}

bool Solver::upload_force_slot() {
    if (!d_force_slot_) return true;
    const ForceSlot f = force_slot();
    CK(cudaMemcpyAsync(d_force_slot_, &f, sizeof f, cudaMemcpyHostToDevice, stream_));
    CK(cudaStreamSynchronize(stream_));
    return true;
}

bool Solver::set_block(dim3 b) {
    block_ = b;
    graph_valid_ = false;
    return true;
}

bool Solver::upload_all_bc_values() {
    for (const Stage &st : stages_) {
        const BCEntry &b = d_.bcs[st.entry];
        if (st.d_val1 && b.val1) CK(cudaMemcpyAsync(st.d_val1, b.val1, st.along * sizeof(double), cudaMemcpyHostToDevice, stream_));
        if (st.d_val2 && b.val2) CK(cudaMemcpyAsync(st.d_val2, b.val2, st.along * sizeof(double), cudaMemcpyHostToDevice, stream_));
    }
    return true;
}

bool Solver::set_bc_values(int entry, const double *val1, const double *val2) {
    for (const Stage &st : stages_) {
        if (st.entry != entry) continue;
        if (st.d_val1 && val1) CK(cudaMemcpyAsync(st.d_val1, val1, st.along * sizeof(double), cudaMemcpyHostToDevice, stream_));
        if (st.d_val2 && val2) CK(cudaMemcpyAsync(st.d_val2, val2, st.along * sizeof(double), cudaMemcpyHostToDevice, stream_));
    }
    return true;
}

bool Solver::set_state(const double *f, const double *f_new, const double *rho, const double *u,
                       const double *v, bool fnew_needed) {
    const int Nx = d_.Nx, Ny = d_.Ny;
    const size_t N = (size_t)Nx * Ny;
    cur_ = 0;
    fields_are_moments_ = false;  // the caller's fields: lbc collides with them as given
    const double *src[2] = {f, f_new};
    for (int b = 0; b < 2; b++) {
        // The drop-in skips f_new when its old content cannot reach the
        // results (no solid nodes, no off-grid pull sources).
        if (b == 1 && !fnew_needed) continue;
        for (int j0 = 0; j0 < Ny; j0 += stage_rows_) {
            const int rows = std::min(stage_rows_, Ny - j0);
            CK(cudaMemcpyAsync(d_stage_, src[b] + (size_t)j0 * Nx * 9, (size_t)rows * Nx * 9 * sizeof(double),
                               cudaMemcpyHostToDevice, stream_));
            CK(launch::aos_to_soa(d_stage_, (char *)buf_[b] + (size_t)j0 * pitch_ * esize_, d_.store, Nx, rows,
                                  pitch_, plane_, d_.w, stream_));
        }
    }
    CK(cudaMemcpyAsync(d_rho_, rho, N * sizeof(double), cudaMemcpyHostToDevice, stream_));
    CK(cudaMemcpyAsync(d_ux_, u, N * sizeof(double), cudaMemcpyHostToDevice, stream_));
    CK(cudaMemcpyAsync(d_uy_, v, N * sizeof(double), cudaMemcpyHostToDevice, stream_));
    if (nslots_ > 0)
        CK(launch::seed_band(d_seed_nodes_, d_seed_slots_, nseed_, Nx, d_rho_, d_ux_, d_uy_,
                             d_bandm_[parity_], nslots_, stream_));
    return true;
}

bool Solver::get_state(double *f, double *f_new, double *rho, double *u, double *v) {
    const int Nx = d_.Nx, Ny = d_.Ny;
    double *dst[2] = {f, f_new};
    const int which[2] = {cur_, 1 - cur_};
    for (int b = 0; b < 2; b++) {
        if (!dst[b]) continue;
        for (int j0 = 0; j0 < Ny; j0 += stage_rows_) {
            const int rows = std::min(stage_rows_, Ny - j0);
            CK(launch::soa_to_aos((const char *)buf_[which[b]] + (size_t)j0 * pitch_ * esize_, d_stage_, d_.store,
                                  Nx, rows, pitch_, plane_, d_.w, stream_));
            CK(cudaMemcpyAsync(dst[b] + (size_t)j0 * Nx * 9, d_stage_, (size_t)rows * Nx * 9 * sizeof(double),
                               cudaMemcpyDeviceToHost, stream_));
        }
    }
    if (!get_fields(rho, u, v)) return false;
    CK(cudaStreamSynchronize(stream_));
    return true;
}

bool Solver::dropin_step_direct(double *f, double *f_new, double *rho, double *u, double *v) {
    if (d_.store != STORE_F64) {
        set_error("direct drop-in step needs FP64 storage");
        return false;
    }
    const int Nx = d_.Nx, Ny = d_.Ny;
    cur_ = 0;
    if (nslots_ > 0)
        CK(launch::seed_band(d_seed_nodes_, d_seed_slots_, nseed_, Nx, rho, u, v, d_bandm_[parity_],
                             nslots_, stream_));
    CollideAosParams c;
    std::memset(&c, 0, sizeof c);
    c.Nx = Nx; c.Ny = Ny; c.pitch = pitch_; c.plane = plane_;
    c.f_aos = f;
    c.soa = (double *)buf_[0];
    c.flags = d_flags_;
    c.rho = rho; c.ux = u; c.uy = v;
    c.omega = d_omega_; c.omega0 = omega0_;
    c.has_force = (d_.Fx != 0.0 || d_.Fy != 0.0);
    c.Fx = d_.Fx; c.Fy = d_.Fy;
    for (int k = 0; k < 9; k++) c.w[k] = d_.w[k];
    CK(launch::collide_aos_exact(c, stream_));
    // Without solid nodes or off-grid pull sources every slot of f_new is
    // rewritten before it is read, so its old content is not needed.
    if (needs_old_dst_)
        CK(launch::aos_to_soa(f_new, buf_[1], STORE_F64, Nx, Ny, pitch_, plane_, d_.w, stream_));
    macro_out_[0] = rho; macro_out_[1] = u; macro_out_[2] = v;
    const bool okk = launch_step(0, 1, false, true, parity_);
    macro_out_[0] = macro_out_[1] = macro_out_[2] = nullptr;
    if (!okk) return false;
    CK(launch::soa_to_aos(buf_[1], f_new, STORE_F64, Nx, Ny, pitch_, plane_, d_.w, stream_));
    cur_ = 1;
    parity_ ^= 1;
    steps_done_ += 1;
    CK(cudaStreamSynchronize(stream_));
    return true;
}

bool Solver::get_fields(double *rho, double *u, double *v) {
    const size_t N = (size_t)d_.Nx * d_.Ny;
    if (rho) CK(cudaMemcpyAsync(rho, d_rho_, N * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    if (u) CK(cudaMemcpyAsync(u, d_ux_, N * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    if (v) CK(cudaMemcpyAsync(v, d_uy_, N * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    return true;
}

bool Solver::forces(double *Fx, double *Fy) {
    double h[2] = {0.0, 0.0};
    if (has_mem_) {
        CK(cudaMemcpyAsync(h, d_mem_out_, 2 * sizeof(double), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
    }
    if (Fx) *Fx = h[0];
    if (Fy) *Fy = h[1];
    return true;
}

bool Solver::enable_force_history(int capacity) {
    if (!has_mem_) {
        set_error("the geometry has no wall links: no force to record");
        return false;
    }
    if (capacity <= 0) {
        set_error("force history capacity must be positive");
        return false;
    }
    if (!dalloc(&d_hist_, (size_t)capacity * 2)) return false;
    unsigned long long *cnt = nullptr;
    if (!dalloc(&cnt, 1)) return false;
    CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), stream_));
    hist_cap_ = capacity;
    hist_count_ptr_ = cnt;
    hist_written_ = 0;  // a new ring: its records count from its first step
    graph_valid_ = false;
    return upload_force_slot();
}

int Solver::force_history(double *out, int max_steps) {
    if (!d_hist_) return 0;
    unsigned long long cnt = 0;
    if (!check_cuda(cudaMemcpyAsync(&cnt, hist_count_ptr_, sizeof cnt, cudaMemcpyDeviceToHost, stream_), "history"))
        return -1;
    if (!check_cuda(cudaStreamSynchronize(stream_), "history")) return -1;
    const long long avail = std::min<long long>((long long)cnt, hist_cap_);
    const int n = (int)std::min<long long>(avail, max_steps);
    // Oldest first.
    std::vector<double> ring((size_t)hist_cap_ * 2);
    if (!check_cuda(cudaMemcpy(ring.data(), d_hist_, ring.size() * sizeof(double), cudaMemcpyDeviceToHost), "history"))
        return -1;
    const long long first = (long long)cnt - n;
    for (int s = 0; s < n; s++) {
        const long long slot = (first + s) % hist_cap_;
        out[2 * s] = ring[2 * slot];
        out[2 * s + 1] = ring[2 * slot + 1];
    }
    return n;
}

// lbc's force record file (cases/cylinder/cylinder.c:162-185): per step n
// (counted from lbm_gpu_enable_force_history) three doubles, n * dt, L * cf,
// D * cf, in the host's byte order, written with one fwrite each as lbc does.
long long Solver::write_force_records(const char *path, double dt, double cf, bool append) {
    if (!d_hist_) {
        set_error("force history is not enabled");
        return -1;
    }
    unsigned long long cnt = 0;
    std::vector<double> ring((size_t)hist_cap_ * 2);
    if (!check_cuda(cudaMemcpyAsync(&cnt, hist_count_ptr_, sizeof cnt, cudaMemcpyDeviceToHost, stream_), "records") ||
        !check_cuda(cudaMemcpyAsync(ring.data(), d_hist_, ring.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                    stream_), "records") ||
        !check_cuda(cudaStreamSynchronize(stream_), "records"))
        return -1;
    FILE *fp = std::fopen(path, append ? "ab" : "wb");
    if (!fp) {
        set_error(std::string("cannot open ") + path);
        return -1;
    }
    // Steps older than the ring's capacity are gone: write from the oldest held.
    const unsigned long long first = std::max<unsigned long long>(
        hist_written_, cnt > (unsigned long long)hist_cap_ ? cnt - hist_cap_ : 0);
    const bool lost = first > hist_written_;
    struct Record { double time, L, D; };
    bool okk = true;
    for (unsigned long long n = first; n < cnt && okk; n++) {
        const size_t slot = (size_t)(n % (unsigned long long)hist_cap_);
        const Record rec{(double)n * dt, ring[2 * slot + 1] * cf, ring[2 * slot] * cf};
        okk = std::fwrite(&rec, sizeof rec, 1, fp) == 1;
    }
    okk = (std::fclose(fp) == 0) && okk;
    if (!okk) {
        set_error(std::string("write failed: ") + path);
        return -1;
    }
    const unsigned long long missed = first - hist_written_;
    hist_written_ = std::max(hist_written_, cnt);
    if (lost) {
        set_error("the force records of " + std::to_string(missed) +
                  " steps left the ring before they were written (drain it at least every capacity steps)");
        return -2;
    }
    return first < cnt ? (long long)(cnt - first) : 0;
}

bool Solver::launch_collide(int b, cudaStream_t s) {
    if (!s) s = stream_;
    CollideParams c;
    c.Nx = d_.Nx; c.Ny = d_.Ny; c.pitch = pitch_; c.plane = plane_;
    c.f = (double *)buf_[b];
    c.flags = d_flags_;
    c.rho = d_rho_; c.ux = d_ux_; c.uy = d_uy_;
    c.omega = d_omega_; c.omega0 = omega0_;
    c.has_force = (d_.Fx != 0.0 || d_.Fy != 0.0);
    c.Fx = d_.Fx; c.Fy = d_.Fy;
    for (int k = 0; k < 9; k++) c.w[k] = d_.w[k];
    c.from_pops = fields_are_moments_ ? 1 : 0;
    c.fma = d_.fma64 ? 1 : 0;
    if (d_.store == STORE_F64) CK(launch::collide_exact(c, s));
    else CK(launch::collide_shifted(c, d_.store, s));
    return true;
}

StepParams Solver::step_params(int src, int dst, bool write_macro, int bparity) const {
    StepParams p;
    std::memset(&p, 0, sizeof p);
    p.Nx = d_.Nx; p.Ny = d_.Ny; p.pitch = pitch_; p.plane = plane_;
    p.px = d_.px; p.py = d_.py;
    p.src = buf_[src]; p.dst = buf_[dst];
    p.flags = d_flags_; p.link_off = d_link_off_; p.links = d_links_;
    p.seg_clean = d_seg_clean_; p.seg_words = seg_words_;
    p.omega = d_omega_; p.omega0 = omega0_;
    p.has_force = (d_.Fx != 0.0 || d_.Fy != 0.0);
    p.Fx = d_.Fx; p.Fy = d_.Fy; p.hFx = 0.5 * d_.Fx; p.hFy = 0.5 * d_.Fy;
    for (int k = 0; k < 9; k++) p.w[k] = d_.w[k];
    p.write_macro = write_macro ? 1 : 0;
    p.rho = macro_out_[0] ? macro_out_[0] : d_rho_;
    p.ux = macro_out_[1] ? macro_out_[1] : d_ux_;
    p.uy = macro_out_[2] ? macro_out_[2] : d_uy_;
    p.colbase = d_colbase_; p.rowbase = d_rowbase_; p.nslots = nslots_;
    p.bandf = d_bandf_;
    p.bandg = d_bandg_;
    p.bandm_next = nslots_ ? d_bandm_[bparity ^ 1] : nullptr;
    if (has_mem_) {
        p.mem_partials = d_partials_;
        if (d_.store == STORE_F64) p.seg_slot = d_seg_slot_;
        else p.chunk_slot = d_seg_slot_;
    }
    return p;
}

FastStepParams Solver::fast_params(const StepParams &p) const {
    FastStepParams fp;
    std::memset(&fp, 0, sizeof fp);
    fp.s = p;
    for (int k = 0; k < 9; k++) fp.wf[k] = (float)d_.w[k];
    fp.omega0f = (float)omega0_;
    fp.Fxf = (float)d_.Fx; fp.Fyf = (float)d_.Fy;
    fp.hFxf = (float)(0.5 * d_.Fx); fp.hFyf = (float)(0.5 * d_.Fy);
    fp.h1f = 3.0f * fp.wf[1];
    fp.h5f = (1.0f - 2.0f * fp.h1f) * 0.25f;
    return fp;
}

StageParams Solver::stage_params(const Stage &st, int src, int bparity) const {
    StageParams s;
    std::memset(&s, 0, sizeof s);
    s.Nx = d_.Nx; s.Ny = d_.Ny; s.pitch = pitch_; s.plane = plane_;
    s.kind = st.kind; s.index = st.index; s.along = st.along;
    s.val1 = st.d_val1; s.val2 = st.d_val2;
    s.flags = d_flags_; s.colbase = d_colbase_; s.rowbase = d_rowbase_; s.nslots = nslots_;
    s.bandf = d_bandf_; s.bandg = d_bandg_; s.bandm_prev = d_bandm_[bparity];
    s.src = buf_[src];
    for (int k = 0; k < 9; k++) {
        s.w[k] = d_.w[k];
        s.wf[k] = (float)d_.w[k];
    }
    s.last = d_last_;
    s.entry = (int)(&st - stages_.data());
    s.imp = st.d_imp;
    s.imp_nf = st.imp_nf;
    s.imp_alpha = st.imp_alpha;
    s.imp_wcos = st.imp_wcos;
    s.imp_wsin = st.imp_wsin;
    s.imp_windowed = st.imp_windowed;
    s.imp_slot = bparity;
    for (int f = 0; f < 8; f++) {
        s.imp_cos[f] = st.imp_cos[f];
        s.imp_sin[f] = st.imp_sin[f];
    }
    return s;
}

bool msd_zoh(double R, double m, double K, double A[4], double b[2]) {
    if (!(m > 0.0) || !(K > 0.0) || !(R >= 0.0)) return false;
    // M = [[0, 1], [-K/m, -R/m]]; exp(M) = E0 I + E1 (M - a I), a = tr/2,
    // d^2 = a^2 - det; e^a cosh d and e^a sinh(d)/d formed from e^(a +- d)
    // so that strongly damped nodes do not overflow.
    const double km = K / m, rm = R / m;
    const double a = -0.5 * rm;
    const double d2 = a * a - km;
    double E0, E1;
    if (d2 > 0.0) {
        const double d = std::sqrt(d2);
        const double ep = std::exp(a + d), em = std::exp(a - d);
        E0 = 0.5 * (ep + em);
        E1 = 0.5 * (ep - em) / d;
    } else if (d2 < 0.0) {
        const double wd = std::sqrt(-d2);
        const double ea = std::exp(a);
        E0 = ea * std::cos(wd);
        E1 = ea * std::sin(wd) / wd;
    } else {
        E0 = std::exp(a);
        E1 = std::exp(a);
    }
    A[0] = E0 + E1 * (0.0 - a);  // A11
    A[1] = E1 * 1.0;             // A12
    A[2] = E1 * (-km);           // A21
    A[3] = E0 + E1 * (-rm - a);  // A22
    // b = M^-1 (A - I) (0, 1/m); det M = K/m.
    const double q1 = A[1] / m, q2 = (A[3] - 1.0) / m;
    b[0] = (-rm * q1 - q2) / km;
    b[1] = q1;
    return true;
}

bool Solver::set_impedance(int entry, const double *R, const double *m, const double *K, int nf,
                           const double *omegas, double rho_ref, double alpha, int window) {
    Stage *st = nullptr;
    for (Stage &x : stages_)
        if (x.entry == entry) st = &x;
    if (!st || st->kind != BC_VEL_BOT_REG) {
        set_error("impedance wall: entry must be a velocity_bottom_regularized Boundary entry");
        return false;
    }
    if (!(alpha >= 0.0 && alpha < 1.0)) {
        set_error("impedance wall: alpha must be in [0, 1)");
        return false;
    }
    if (nf < 0 || nf > 8) {
        set_error("impedance wall: at most 8 DFT frequencies");
        return false;
    }
    const int n = st->along;
    std::vector<double> h(imp_doubles(nf, n), 0.0);
    // Both slots of the phasor table start at n = 0: window phasor (1, 0),
    // e^{-i w 0} = (1, 0) per frequency.
    for (int slot = 0; slot < 2; slot++) {
        double *tab = h.data() + imp_tab_offset(nf, n, slot);
        tab[0] = 1.0;
        for (int f = 0; f < nf; f++) tab[2 + 2 * f] = 1.0;
    }
    for (int t = 0; t < n; t++) {
        if (!(m[t] > 0.0)) continue;
        double A[4], b[2];
        if (!msd_zoh(R[t], m[t], K[t], A, b)) {
            set_error("impedance wall: need m > 0, K > 0, R >= 0 at node " + std::to_string(t));
            return false;
        }
        h[(size_t)IMP_ACTIVE * n + t] = 1.0;
        h[(size_t)IMP_A11 * n + t] = A[0];
        h[(size_t)IMP_A12 * n + t] = A[1];
        h[(size_t)IMP_A21 * n + t] = A[2];
        h[(size_t)IMP_A22 * n + t] = A[3];
        h[(size_t)IMP_B1 * n + t] = b[0];
        h[(size_t)IMP_B2 * n + t] = b[1];
        h[(size_t)IMP_RHOBAR * n + t] = rho_ref;
    }
    if (!st->d_imp || st->imp_nf != nf) {
        if (!dalloc(&st->d_imp, h.size())) return false;
    }
    CK(cudaMemcpyAsync(st->d_imp, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, stream_));
    CK(cudaStreamSynchronize(stream_));
    st->imp_nf = nf;
    st->imp_alpha = alpha;
    st->imp_windowed = window > 0 ? 1 : 0;
    st->imp_wcos = window > 0 ? std::cos(2.0 * M_PI / window) : 1.0;
    st->imp_wsin = window > 0 ? std::sin(2.0 * M_PI / window) : 0.0;
    for (int f = 0; f < nf; f++) {
        st->imp_cos[f] = std::cos(omegas[f]);
        st->imp_sin[f] = std::sin(omegas[f]);
    }
    graph_valid_ = false;
    // a wall trace reads this array: its record task follows a new allocation
    return st->d_trace ? upload_records() : true;
}

bool Solver::impedance_readback(int entry, double *out, double *state) {
    const Stage *st = nullptr;
    for (const Stage &x : stages_)
        if (x.entry == entry) st = &x;
    if (!st || !st->d_imp) {
        set_error("impedance wall: none on this entry");
        return false;
    }
    const int n = st->along, nf = st->imp_nf;
    std::vector<double> h((size_t)(IMP_FIELDS + 4 * nf) * n);
    CK(cudaStreamSynchronize(stream_));
    CK(cudaMemcpy(h.data(), st->d_imp, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int t = 0; t < n; t++) {
        if (state) {
            state[2 * t] = h[(size_t)IMP_X * n + t];
            state[2 * t + 1] = h[(size_t)IMP_V * n + t];
        }
        if (out)
            for (int f = 0; f < nf; f++)
                for (int q = 0; q < 4; q++) out[((size_t)t * nf + f) * 4 + q] = h[(size_t)imp_field(f, q) * n + t];
    }
    return true;
}

FinishParams Solver::finish_params(int dst, bool write_macro, int bparity) const {
    FinishParams f;
    std::memset(&f, 0, sizeof f);
    f.Nx = d_.Nx; f.Ny = d_.Ny; f.pitch = pitch_; f.plane = plane_;
    f.colbase = d_colbase_; f.rowbase = d_rowbase_; f.nslots = nslots_;
    f.bandf = d_bandf_; f.bandg = d_bandg_; f.bandm_next = nslots_ ? d_bandm_[bparity ^ 1] : nullptr;
    f.dst = buf_[dst];
    f.omega = d_omega_; f.omega0 = omega0_;
    f.has_force = (d_.Fx != 0.0 || d_.Fy != 0.0);
    f.Fx = d_.Fx; f.Fy = d_.Fy; f.hFx = 0.5 * d_.Fx; f.hFy = 0.5 * d_.Fy;
    for (int k = 0; k < 9; k++) {
        f.w[k] = d_.w[k];
        f.wf[k] = (float)d_.w[k];
    }
    f.omega0f = (float)omega0_;
    f.Fxf = (float)d_.Fx; f.Fyf = (float)d_.Fy;
    f.hFxf = (float)f.hFx; f.hFyf = (float)f.hFy;
    f.write_macro = write_macro ? 1 : 0;
    f.rho = macro_out_[0] ? macro_out_[0] : d_rho_;
    f.ux = macro_out_[1] ? macro_out_[1] : d_ux_;
    f.uy = macro_out_[2] ? macro_out_[2] : d_uy_;
    return f;
}

// One time step src -> dst: fused bulk kernel, then the Boundary list in order,
// one launch per stage group, whose threads finish the BC-written nodes.
bool Solver::launch_step_kernels(int src, int dst, bool collide, bool write_macro, int bparity,
                                 cudaStream_t s) {
    if (!s) s = stream_;
    // The wall force is needed on a step that writes the fields (a run's
    // last step: lbm_gpu_forces reports it) and on every step of a force
    // history; other steps store no force partials and reduce none.
    const bool forces = has_mem_ && (write_macro || hist_cap_ > 0);
    StepParams p = step_params(src, dst, write_macro, bparity);
    if (!forces) p.mem_partials = nullptr;
    if (d_.store == STORE_F64) {
        CK(launch::step_exact(p, has_flags_, collide, block_, s, d_.fma64));
    } else {
        const FastStepParams fp = fast_params(p);
        // The special nodes first, as an ordinary launch, then the clean pairs
        // as its programmatic follower: the grid of clean-pair blocks fills the
        // SMs around the special nodes' latency-bound blocks from the start
        // (the plain kernel of a flag-free grid steps its own odd column).
        // What follows is an ordinary launch, so it sees both.
        if (special_launch()) CK(launch::special_shifted(fp, d_special_, nspecial_, d_.store, true, collide, false, s));
        CK(launch::step_shifted(fp, d_.store, has_flags_, collide, block_, s, special_launch()));
    }
    const bool after_bulk = d_.store == STORE_F64;
    if (groups_.empty()) {
        if (forces) CK(launch::force_reduce(d_force_slot_, 1, after_bulk, s));
        return true;
    }
    // The force (from the bulk kernel's partials) rides in the first stage
    // launch; fused stages finish their nodes (group_stages).
    const FinishParams f = finish_params(dst, write_macro, bparity);
    for (size_t gi = 0; gi < groups_.size(); gi++) {
        const std::vector<int> &g = groups_[gi];
        StageGroup sg;
        std::memset(&sg, 0, sizeof sg);
        sg.n = (int)g.size();
        for (int q = 0; q < sg.n; q++) {
            sg.p[q] = stage_params(stages_[g[q]], src, bparity);
            sg.max_along = std::max(sg.max_along, sg.p[q].along);
        }
        sg.fin = f;
        sg.fs = d_force_slot_;
        sg.nfs = (gi == 0 && forces) ? 1 : 0;
        sg.warm = (long long)d_.Nx * d_.Ny < (1LL << 20) ? 1 : 0;
        CK(launch::stage_group(sg, d_.store, collide, gi == 0 && after_bulk, s));
    }
    return true;
}

// One step (launch_step_kernels), then its records when probes or wall
// traces are set: they read what the step's kernels left, so they follow them.
bool Solver::launch_step(int src, int dst, bool collide, bool write_macro, int bparity, cudaStream_t s) {
    if (!launch_step_kernels(src, dst, collide, write_macro, bparity, s)) return false;
    if (!rec_host_.empty())
        CK(launch::record(d_rec_, (int)rec_host_.size(), d_.store, buf_[dst], nullptr, 0, 0, collide,
                          s ? s : stream_));
    return true;
}

bool Solver::upload_records() {
    rec_host_.clear();
    if (nprobes_ > 0) {
        RecordTask r;
        std::memset(&r, 0, sizeof r);
        r.kind = REC_PROBES;
        r.n = nprobes_;
        r.cs = -1;
        r.cap = probe_cap_;
        r.nodes = d_probe_nodes_;
        r.plane = plane_;
        r.ring = d_probe_ring_;
        r.count = probe_count_;
        for (int k = 0; k < 9; k++) r.w[k] = d_.w[k];
        r.hFx = 0.5 * d_.Fx;
        r.hFy = 0.5 * d_.Fy;
        rec_host_.push_back(r);
    }
    for (const Stage &st : stages_) {
        if (!st.d_trace || !st.d_imp) continue;
        RecordTask r;
        std::memset(&r, 0, sizeof r);
        r.kind = REC_WALL;
        r.n = st.along;
        r.cs = -1;
        r.cap = st.trace_cap;
        r.imp = st.d_imp;
        r.ring = st.d_trace;
        r.count = st.trace_count;
        rec_host_.push_back(r);
    }
    graph_valid_ = false;
    if (rec_host_.empty()) return true;
    if ((int)rec_host_.size() > rec_cap_) {
        if (!dalloc(&d_rec_, rec_host_.size())) return false;
        rec_cap_ = (int)rec_host_.size();
    }
    CK(cudaMemcpyAsync(d_rec_, rec_host_.data(), rec_host_.size() * sizeof(RecordTask), cudaMemcpyHostToDevice,
                       stream_));
    CK(cudaStreamSynchronize(stream_));
    return true;
}

bool Solver::set_probes(int n, const int *pi, const int *pj, int capacity) {
    if (n < 0 || n > kMaxProbes || (n > 0 && (!pi || !pj || capacity <= 0))) {
        set_error("probes: need 0 <= n <= " + std::to_string(kMaxProbes) + ", node arrays and capacity > 0");
        return false;
    }
    std::vector<long long> off((size_t)n);
    for (int q = 0; q < n; q++) {
        if (pi[q] < 0 || pi[q] >= d_.Nx || pj[q] < 0 || pj[q] >= d_.Ny) {
            set_error("probes: node " + std::to_string(q) + " is outside the grid");
            return false;
        }
        off[q] = (long long)pj[q] * pitch_ + pi[q];
    }
    nprobes_ = 0;
    if (n > 0) {
        if (!dalloc(&d_probe_nodes_, (size_t)n) || !dalloc(&d_probe_ring_, (size_t)capacity * n * 3) ||
            !dalloc(&probe_count_, 1))
            return false;
        CK(cudaMemcpyAsync(d_probe_nodes_, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice,
                           stream_));
        CK(cudaMemsetAsync(probe_count_, 0, sizeof(unsigned long long), stream_));
        nprobes_ = n;
        probe_cap_ = capacity;
    }
    return upload_records();
}

int Solver::probe_history(double *out, int max_steps) {
    if (nprobes_ == 0) return 0;
    unsigned long long cnt = 0;
    std::vector<double> ring((size_t)probe_cap_ * nprobes_ * 3);
    if (!check_cuda(cudaMemcpyAsync(&cnt, probe_count_, sizeof cnt, cudaMemcpyDeviceToHost, stream_), "probes") ||
        !check_cuda(cudaMemcpyAsync(ring.data(), d_probe_ring_, ring.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                    stream_), "probes") ||
        !check_cuda(cudaStreamSynchronize(stream_), "probes"))
        return -1;
    const long long avail = std::min<long long>((long long)cnt, probe_cap_);
    const int n = (int)std::min<long long>(avail, max_steps);
    const long long first = (long long)cnt - n;
    const size_t rec = (size_t)nprobes_ * 3;
    for (int t = 0; t < n; t++) {
        const size_t slot = (size_t)((first + t) % probe_cap_);
        std::memcpy(out + (size_t)t * rec, ring.data() + slot * rec, rec * sizeof(double));
    }
    return n;
}

bool Solver::enable_impedance_trace(int entry, int capacity) {
    Stage *st = nullptr;
    for (Stage &x : stages_)
        if (x.entry == entry) st = &x;
    if (!st || !st->d_imp) {
        set_error("impedance trace: no impedance wall on this entry");
        return false;
    }
    if (capacity <= 0) {
        set_error("impedance trace: capacity must be positive");
        return false;
    }
    if (!dalloc(&st->d_trace, (size_t)capacity * 2) || !dalloc(&st->trace_count, 1)) return false;
    CK(cudaMemsetAsync(st->trace_count, 0, sizeof(unsigned long long), stream_));
    st->trace_cap = capacity;
    st->trace_written = 0;
    return upload_records();
}

// lbc's trace of its impedance BC (cases/nit/nit.c:262-273): a text line
// "%lf %lf %lf\n" per iteration, time, surface-averaged pressure fluctuation
// and acoustic velocity, where the line of iteration n holds the values
// computed in iteration n - 1 (the file starts with a line of zeros). Here the
// values of step n are the wall's mean p' and v over its active nodes
// (scaled by cp and cu to physical units), the time (n + 1) dt. Lines not
// written yet are appended (append) or the file is started.
long long Solver::write_impedance_trace(int entry, const char *path, double dt, double cp, double cu,
                                        bool append) {
    Stage *st = nullptr;
    for (Stage &x : stages_)
        if (x.entry == entry) st = &x;
    if (!st || !st->d_trace) {
        set_error("impedance trace: not enabled on this entry");
        return -1;
    }
    unsigned long long cnt = 0;
    std::vector<double> ring((size_t)st->trace_cap * 2);
    if (!check_cuda(cudaMemcpyAsync(&cnt, st->trace_count, sizeof cnt, cudaMemcpyDeviceToHost, stream_), "trace") ||
        !check_cuda(cudaMemcpyAsync(ring.data(), st->d_trace, ring.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                    stream_), "trace") ||
        !check_cuda(cudaStreamSynchronize(stream_), "trace"))
        return -1;
    FILE *fp = std::fopen(path, append ? "a" : "w");
    if (!fp) {
        set_error(std::string("cannot open ") + path);
        return -1;
    }
    const unsigned long long first = std::max<unsigned long long>(
        st->trace_written, cnt > (unsigned long long)st->trace_cap ? cnt - st->trace_cap : 0);
    const bool lost = first > st->trace_written;
    bool okk = true;
    long long lines = 0;
    if (st->trace_written == 0 && !append) {
        okk = std::fprintf(fp, "%lf %lf %lf\n", 0.0, 0.0, 0.0) > 0;
        lines++;
    }
    for (unsigned long long n = first; n < cnt && okk; n++) {
        const size_t slot = (size_t)(n % (unsigned long long)st->trace_cap);
        okk = std::fprintf(fp, "%lf %lf %lf\n", (double)(n + 1) * dt, ring[2 * slot] * cp, ring[2 * slot + 1] * cu) > 0;
        lines++;
    }
    okk = (std::fclose(fp) == 0) && okk;
    if (!okk) {
        set_error(std::string("write failed: ") + path);
        return -1;
    }
    const unsigned long long missed = first - st->trace_written;
    st->trace_written = std::max(st->trace_written, cnt);
    if (lost) {
        set_error("the trace of " + std::to_string(missed) +
                  " steps left the ring before it was written (drain it at least every capacity steps)");
        return -2;
    }
    return lines;
}

bool Solver::begin_steps(cudaStream_t s) { return launch_collide(cur_, s); }

bool Solver::end_steps(cudaStream_t s) {
    if (!launch_step(cur_, 1 - cur_, false, true, parity_, s)) return false;
    advance(1);
    fields_are_moments_ = true;
    return true;
}

void Solver::advance(int nsteps) {
    if (nsteps & 1) {
        cur_ ^= 1;
        parity_ ^= 1;
    }
}

// Two fused steps (cur -> other -> cur) captured once and replayed.
bool Solver::capture_pair() {
    if (graph_valid_ && pair_cur_ == cur_ && pair_parity_ == parity_) return true;
    if (pair_exec_) {
        cudaGraphExecDestroy(pair_exec_);
        pair_exec_ = nullptr;
    }
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    bool okk = launch_step(cur_, 1 - cur_, true, false, parity_) &&
               launch_step(1 - cur_, cur_, true, false, parity_ ^ 1);
    cudaError_t e = cudaStreamEndCapture(stream_, &g);
    if (!okk) {
        if (g) cudaGraphDestroy(g);
        return false;
    }
    CK(e);
    e = cudaGraphInstantiate(&pair_exec_, g, 0);
    cudaGraphDestroy(g);
    CK(e);
    pair_cur_ = cur_;
    pair_parity_ = parity_;
    graph_valid_ = true;
    return true;
}

// This case's tiles for the batched kernel (x = 0, y = x0, z = y0, w = 1 when
// the tile contains wall links), built once per tile shape: the batch
// concatenates them instead of rescanning every node whenever it is rebuilt.
const std::vector<int4> &Solver::tiles(int tws) const {
    const int key = tws;
    auto it = tile_cache_.find(key);
    if (it != tile_cache_.end()) return it->second;
    std::vector<int4> out;
    const int Nx = d_.Nx, Ny = d_.Ny;
    const int tw = (d_.store == STORE_F64 ? 1 : 2) << tws, th = 256 >> tws;
    for (int y = 0; y < Ny; y += th)
        for (int x = 0; x < Nx; x += tw) {
            int w = 0;
            if (has_mem_) {
                for (int j = y; j < std::min(Ny, y + th) && !w; j++)
                    for (int i = x; i < std::min(Nx, x + tw); i++)
                        if (link_node_[(size_t)j * Nx + i]) { w = 1; break; }
            }
            out.push_back(make_int4(0, x, y, w));
        }
    return tile_cache_.emplace(key, std::move(out)).first->second;
}

std::string Solver::tune_key() const {
    return device_tag() + "/step/s" + std::to_string(storage_code()) + "/" + std::to_string(d_.Nx) + "x" +
           std::to_string(d_.Ny) + (has_flags_ ? "/geo" : "/plain") + (has_mem_ ? "/mem" : "");
}

void Solver::set_autotune(int mode) {
    tune_mode_ = mode ? 1 : 0;
    tuned_ = false;
    tuned_us_ = 0.f;
    if (!tune_mode_) return;
    int bx = 0, by = 0;
    if (tune_lookup(tune_key(), bx, by) && bx >= 32 && bx % 32 == 0 && by >= 1 && bx * by <= 256) {
        set_block(dim3(bx, by, 1));
        tuned_ = true;
    }
}

// One fused step cur -> other, as inside run().
bool Solver::trial_step() {
    if (!launch_step(cur_, 1 - cur_, true, false, parity_)) return false;
    cur_ ^= 1;
    parity_ ^= 1;
    return true;
}

// Candidate blocks of the fused step: warp-wide rows (bx a multiple of 32),
// 64 to 256 threads.
static const int kBlockCand[][2] = {{64, 4}, {32, 8}, {128, 2}, {256, 1}, {32, 4}, {64, 2}, {128, 1}};
static const int kNBlockCand = 7;

// Times each candidate block over two interleaved windows of K real steps
// (after two steps that estimate K) and keeps the fastest. Returns the number
// of steps taken (all of them steps of the run), or -1 on a CUDA error.
int Solver::tune_online(int avail) {
    const int nc = kNBlockCand;
    WindowTimer est(1);
    if (!est.ok()) return -1;
    if (!est.mark(0, stream_) || !trial_step() || !trial_step() || !est.mark(1, stream_) || !est.wait()) return -1;
    int used = 2;
    int K = window_steps(est.elapsed(0) / 2.f, 0.25f, 2, 64);
    K = std::min(K, (avail - used) / (2 * nc));
    if (K < 1) return used;
    WindowTimer wt(2 * nc);
    if (!wt.ok()) return -1;
    for (int r = 0; r < 2; r++)
        for (int c = 0; c < nc; c++) {
            if (!wt.mark(r * nc + c, stream_)) return -1;
            set_block(dim3(kBlockCand[c][0], kBlockCand[c][1], 1));
            for (int k = 0; k < K; k++)
                if (!trial_step()) return -1;
        }
    if (!wt.mark(2 * nc, stream_) || !wt.wait()) return -1;
    used += 2 * nc * K;
    int best = -1;
    float best_ms = 0.f;
    for (int c = 0; c < nc; c++) {
        const float ms = std::min(wt.elapsed(c), wt.elapsed(nc + c));
        if (best < 0 || ms < best_ms) { best = c; best_ms = ms; }
    }
    set_block(dim3(kBlockCand[best][0], kBlockCand[best][1], 1));
    tuned_ = true;
    tuned_us_ = best_ms * 1e3f / K;
    tune_store(tune_key(), kBlockCand[best][0], kBlockCand[best][1], tuned_us_);
    return used;
}

bool Solver::run(int nsteps) {
    if (nsteps <= 0) return true;
    if (!launch_collide(cur_)) return false;
    int remaining = nsteps - 1;
    // Tuning takes its trial windows from the steps of this run.
    if (tune_mode_ && !tuned_ && remaining >= 2 + 2 * kNBlockCand) {
        const int used = tune_online(remaining);
        if (used < 0) return false;
        remaining -= used;
    }
    if (remaining >= 2) {
        if (!capture_pair()) return false;
        while (remaining >= 2) {
            CK(cudaGraphLaunch(pair_exec_, stream_));
            remaining -= 2;
        }
    }
    if (remaining == 1) {
        if (!launch_step(cur_, 1 - cur_, true, false, parity_)) return false;
        cur_ ^= 1;
        parity_ ^= 1;
    }
    if (!launch_step(cur_, 1 - cur_, false, true, parity_)) return false;
    cur_ ^= 1;
    parity_ ^= 1;
    steps_done_ += nsteps;
    fields_are_moments_ = true;
    return true;
}

}  // namespace lbm

// ===================================================================== Batch

namespace lbm {

Batch::Batch(const std::vector<Solver *> &cases) : cases_(cases) {
    if (cases_.empty()) {
        set_error("empty batch");
        return;
    }
    store_ = cases_[0]->store();
    for (Solver *c : cases_) {
        if (!c || !c->ok()) {
            set_error("batch: invalid case");
            return;
        }
        if (c->store() != store_ || c->fma64() != cases_[0]->fma64()) {
            set_error("batch: all cases must use the same storage");
            return;
        }
    }
    // FP64 batches (FP64-issue bound, long) run at the lowest stream priority,
    // shifted-storage batches at the highest, so that when both run at once
    // (the server's lanes) free SMs go to the short, memory-bound FP32 steps
    // (measured the other way round on the 2,000-request stream: p50 104 s
    // instead of 1.2 s, p99 167 instead of 150 s).
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (!check_cuda(cudaStreamCreateWithPriority(&stream_, cudaStreamNonBlocking, store_ == STORE_F64 ? lo : hi),
                    "cudaStreamCreateWithPriority"))
        return;
    ok_ = build();
    if (ok_) set_autotune(tune_default_mode());
}

Batch::~Batch() {
    if (pair_exec_) cudaGraphExecDestroy(pair_exec_);
    if (params_ev_) {
        cudaEventSynchronize(params_ev_);
        cudaEventDestroy(params_ev_);
    }
    if (d_tiles_) cudaFreeAsync(d_tiles_, stream_);
    for (void *p : allocs_) cudaFreeAsync(p, stream_);
    if (stream_) cudaStreamDestroy(stream_);
}

template <class T> static bool balloc(std::vector<void *> &allocs, T **p, size_t n, cudaStream_t s) {
    void *q = nullptr;
    if (!device_alloc(&q, std::max<size_t>(n, 1) * sizeof(T), s)) return false;
    allocs.push_back(q);
    *p = (T *)q;
    return true;
}

// Static tables (tile list, stage entry lists, finish nodes, force slots) and
// room for the per-direction parameter arrays, which run() refreshes.
// Tiles of 2^tws x 2^(8 - tws) threads over every case (one node per thread in
// FP64, two adjacent nodes in shifted storage); w = 1 for tiles that contain
// wall links (their threads store force partials).
std::vector<int4> Batch::make_tiles(int tws) const {
    std::vector<int4> tiles;
    for (int c = 0; c < (int)cases_.size(); c++)
        for (const int4 &t : cases_[c]->tiles(tws))
            tiles.push_back(make_int4(c, t.y, t.z, t.w));
    return tiles;
}

bool Batch::upload_tiles(const std::vector<int4> &tiles, int4 **d) {
    *d = nullptr;
    if (!device_alloc((void **)d, std::max<size_t>(tiles.size(), 1) * sizeof(int4), stream_)) return false;
    CK(cudaMemcpyAsync(*d, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, stream_));
    return true;
}

// Makes (d, n, tws) the tile list of the bulk kernel, freeing the previous
// list when free_old is set (the caller has synchronized the stream).
void Batch::install_tiles(int4 *d, int n, int tws, bool free_old) {
    if (free_old && d_tiles_ && d_tiles_ != d) cudaFreeAsync(d_tiles_, stream_);
    d_tiles_ = d;
    ntiles_ = n;
    tws_ = tws;
    grid_ = std::min(ntiles_, store_ == STORE_F64 ? launch::step_batch_exact_grid()
                                                  : launch::step_batch_shifted_grid(store_));
    if (grid_ < 1) grid_ = 1;
    if (pair_exec_) {
        cudaGraphExecDestroy(pair_exec_);
        pair_exec_ = nullptr;
    }
}

bool Batch::build_tiles(int tws) {
    const std::vector<int4> tiles = make_tiles(tws);
    int4 *d = nullptr;
    CK(cudaStreamSynchronize(stream_));
    if (!upload_tiles(tiles, &d)) return false;
    CK(cudaStreamSynchronize(stream_));
    install_tiles(d, (int)tiles.size(), tws, true);
    return true;
}

std::string Batch::tune_key() const {
    // The composition: each case's grid and geometry class, in order.
    std::string comp;
    for (Solver *c : cases_)
        comp += std::to_string(c->Nx()) + "x" + std::to_string(c->Ny()) + (c->has_flags() ? "g" : "p") +
                (c->has_mem() ? "m" : "") + ",";
    const size_t h = std::hash<std::string>{}(comp);
    char hex[32];
    std::snprintf(hex, sizeof hex, "%016zx", h);
    return device_tag() + "/batch/s" + std::to_string(store_) + "/n" + std::to_string(cases_.size()) + "/" + hex;
}

void Batch::set_autotune(int mode) {
    tune_mode_ = mode ? 1 : 0;
    tuned_ = false;
    tuned_us_ = 0.f;
    if (!tune_mode_) return;
    int tw = 0, th = 0;
    if (tune_lookup(tune_key(), tw, th) && tw * th == 256 && tw >= 32 && (tw & (tw - 1)) == 0) {
        int tws = 0;
        while ((1 << tws) < tw) tws++;
        if (set_tile_shift(tws)) tuned_ = true;
    }
}

static const int kTileCand[] = {6, 5, 7, 8};
static const int kNTileCand = 4;

// As Solver::tune_online, over step pairs of the batched loop (the directions
// of a pair are sel 0 then 1, as in the captured graph). Returns the pairs taken.
int Batch::tune_online(int avail_pairs) {
    const int nc = kNTileCand;
    std::vector<int4 *> d(nc, nullptr);
    std::vector<int> n(nc, 0);
    bool okk = true;
    for (int c = 0; c < nc && okk; c++) {
        const std::vector<int4> t = make_tiles(kTileCand[c]);
        n[c] = (int)t.size();
        okk = upload_tiles(t, &d[c]);
        if (okk) okk = check_cuda(cudaStreamSynchronize(stream_), "sync");
    }
    int4 *const orig = d_tiles_;
    const int orig_n = ntiles_, orig_tws = tws_;
    int used = 0, best = -1;
    float best_ms = 0.f;
    auto pair = [&]() { return launch_batched(0) && launch_batched(1); };
    if (okk) {
        WindowTimer est(1);
        okk = est.ok() && est.mark(0, stream_) && pair() && est.mark(1, stream_) && est.wait();
        used = 1;
        int K = okk ? window_steps(est.elapsed(0), 0.5f, 1, 32) : 0;
        K = std::min(K, (avail_pairs - used) / (2 * nc));
        if (okk && K >= 1) {
            WindowTimer wt(2 * nc);
            okk = wt.ok();
            for (int r = 0; r < 2 && okk; r++)
                for (int c = 0; c < nc && okk; c++) {
                    okk = wt.mark(r * nc + c, stream_);
                    install_tiles(d[c], n[c], kTileCand[c], false);
                    for (int k = 0; k < K && okk; k++) okk = pair();
                }
            okk = okk && wt.mark(2 * nc, stream_) && wt.wait();
            used += 2 * nc * K;
            for (int c = 0; c < nc && okk; c++) {
                const float ms = std::min(wt.elapsed(c), wt.elapsed(nc + c));
                if (best < 0 || ms < best_ms) { best = c; best_ms = ms; }
            }
            if (okk) tuned_us_ = best_ms * 1e3f / (2 * K);
        }
    }
    // Wait for every launch that used a list before freeing the lists not kept.
    cudaStreamSynchronize(stream_);
    if (best >= 0) {
        install_tiles(d[best], n[best], kTileCand[best], false);
        if (orig) cudaFreeAsync(orig, stream_);
        tuned_ = true;
        tune_store(tune_key(), 1 << kTileCand[best], 256 >> kTileCand[best], tuned_us_);
    } else {
        install_tiles(orig, orig_n, orig_tws, false);
    }
    for (int c = 0; c < nc; c++)
        if (d[c] && d[c] != d_tiles_) cudaFreeAsync(d[c], stream_);
    return okk ? used : -1;
}

bool Batch::build() {
    const int nc = (int)cases_.size();
    std::vector<ForceSlot> force;
    for (int c = 0; c < nc; c++) {
        Solver *s = cases_[c];
        nodes_ += (long long)s->Nx() * s->Ny();
        if (9LL * s->plane() >= (1LL << 31)) wide_ = true;
        if (s->has_force()) any_force_ = true;
        if (!s->has_flags()) all_flags_ = false;
        if (s->has_links()) any_links_ = true;
        if (s->has_mem()) force.push_back(s->force_slot());
        max_stages_ = std::max(max_stages_, (int)s->stage_groups().size());
    }
    // Shifted storage: every case's special nodes, each case's list padded to
    // a multiple of 32 so that a warp steps one force chunk of one case. The
    // batched steps write no fields, so marked solids have nothing to do
    // there; runs that reduce no force take a second list without them
    // (chunks then need no owner: on 64 liner ducts 2912 -> 1920 blocks,
    // 184.4 -> 183.0 us per step). A case's own list keeps its row-major
    // order: taking the marked solids out of it scatters the per-node loads
    // of a cylinder's surface over more rows per warp (19.5 -> 20.4 us).
    std::vector<int4> special, special_nf;
    if (store_ != STORE_F64)
        for (int c = 0; c < nc; c++) {
            const std::vector<int2> &sl = cases_[c]->special_nodes();
            const int n = (int)sl.size(), padded = (n + 31) / 32 * 32;
            for (int q = 0; q < padded; q++)
                special.push_back(q < n ? make_int4(c, sl[q].x, sl[q].y, q >> 5) : make_int4(c, -1, -1, q >> 5));
            const size_t first = special_nf.size();
            for (int q = 0; q < n; q++)
                if (!(sl[q].x & kSpecialSolid)) special_nf.push_back(make_int4(c, sl[q].x, sl[q].y, q >> 5));
            while ((special_nf.size() - first) % 32) special_nf.push_back(make_int4(c, -1, -1, 0));
        }
    nspecial_ = (int)special.size();
    nspecial_nf_ = (int)special_nf.size();
    if (!build_tiles(tws_)) return false;
    nforce_ = (int)force.size();
    const size_t psize = store_ == STORE_F64 ? sizeof(StepParams) : sizeof(FastStepParams);
    void *sp = nullptr;
    if (!device_alloc(&sp, psize * 2 * nc, stream_)) return false;
    allocs_.push_back(sp);
    d_sp_ = sp;
    // Entries per stage level (a case may put several stages in one level).
    std::vector<int> level_cnt(max_stages_, 0);
    for (Solver *c : cases_)
        for (size_t l = 0; l < c->stage_groups().size(); l++) level_cnt[l] += (int)c->stage_groups()[l].size();
    if (!balloc(allocs_, &d_fin_, 2 * nc, stream_) || !balloc(allocs_, &d_force_, force.size(), stream_)) return false;
    if (nforce_) CK(cudaMemcpyAsync(d_force_, force.data(), force.size() * sizeof(ForceSlot), cudaMemcpyHostToDevice, stream_));
    if (nspecial_) {
        if (!balloc(allocs_, &d_special_, special.size(), stream_)) return false;
        CK(cudaMemcpyAsync(d_special_, special.data(), special.size() * sizeof(int4), cudaMemcpyHostToDevice, stream_));
    }
    if (nspecial_nf_) {
        if (!balloc(allocs_, &d_special_nf_, special_nf.size(), stream_)) return false;
        CK(cudaMemcpyAsync(d_special_nf_, special_nf.data(), special_nf.size() * sizeof(int4), cudaMemcpyHostToDevice,
                           stream_));
    }
    // One launch per level: level l holds the l-th stage group of every case.
    for (int s = 0; s < max_stages_; s++) {
        const int cnt = level_cnt[s];
        StageParams *d = nullptr;
        if (!balloc(allocs_, &d, 2 * cnt, stream_)) return false;
        d_stage_lists_.push_back(d);
        stage_counts_.push_back(cnt);
    }
    // The blocks of each level's launch: every run of kStageBatchPoints points
    // of an entry with a fluid node, and every entry's first run, whose point
    // 0 advances an impedance wall's window phasor (entries numbered as run()
    // fills the lists); then, on the first level, one block per force slot.
    // (A grid of entries x the longest entry launched 4 to 6 times as many
    // blocks on seeded liner ducts, most of them empty or on the solid wall.)
    {
        const int bs = store_ == STORE_F64 ? launch::kStageBatchPointsF64 : launch::kStageBatchPoints;
        std::vector<int> next(max_stages_, 0);
        std::vector<std::vector<int2>> blocks(max_stages_);
        for (Solver *c : cases_)
            for (size_t l = 0; l < c->stage_groups().size(); l++)
                for (int k : c->stage_groups()[l]) {
                    const Stage &st = c->stages()[k];
                    const int e = next[l]++;
                    for (int t0 = 0; t0 < st.along; t0 += bs) {
                        bool any = t0 == 0;
                        for (int t = t0; t < std::min(st.along, t0 + bs) && !any; t++) any = st.open[t] != 0;
                        if (any) blocks[l].push_back(make_int2(e, t0));
                    }
                }
        if (max_stages_ > 0)
            for (int f = 0; f < nforce_; f++) blocks[0].push_back(make_int2(level_cnt[0] + f, 0));
        for (int l = 0; l < max_stages_; l++) {
            int2 *d = nullptr;
            if (!blocks[l].empty()) {
                if (!balloc(allocs_, &d, blocks[l].size(), stream_)) return false;
                CK(cudaMemcpyAsync(d, blocks[l].data(), blocks[l].size() * sizeof(int2), cudaMemcpyHostToDevice,
                                   stream_));
            }
            d_stage_blocks_.push_back(d);
            stage_nblocks_.push_back((int)blocks[l].size());
        }
    }
    // Every case's probes and wall traces: one record launch per step.
    std::vector<RecordTask> rec;
    for (int c = 0; c < nc; c++)
        for (RecordTask r : cases_[c]->record_tasks()) {
            r.cs = c;
            rec.push_back(r);
        }
    nrec_ = (int)rec.size();
    if (nrec_) {
        if (!balloc(allocs_, &d_rec_, rec.size(), stream_)) return false;
        CK(cudaMemcpyAsync(d_rec_, rec.data(), rec.size() * sizeof(RecordTask), cudaMemcpyHostToDevice, stream_));
    }
    // The force reductions ride in the first stage level's launch.
    int stage_launches = 0;
    for (int nb : stage_nblocks_) stage_launches += nb > 0 ? 1 : 0;
    launches_per_step_ = 1 + (nspecial_ ? 1 : 0) + stage_launches +
                         (nforce_ && max_stages_ == 0 ? 1 : 0) + (nrec_ ? 1 : 0);
    CK(cudaStreamSynchronize(stream_));
    return true;
}

bool Batch::launch_batched(int sel) {
    if (store_ == STORE_F64) {
        CK(launch::step_batch_exact((const StepParams *)d_sp_, d_tiles_, ntiles_, sel, tws_,
                                    grid_, stream_, cases_[0]->fma64()));
    } else {
        // the clean pairs, then the special nodes overlapping their tail
        CK(launch::step_batch_shifted((const FastStepParams *)d_sp_, d_tiles_, ntiles_, sel, tws_,
                                      store_, wide_, any_force_, all_flags_, grid_, stream_));
        CK(launch::special_batch_shifted((const FastStepParams *)d_sp_, forces_ ? d_special_ : d_special_nf_,
                                         forces_ ? nspecial_ : nspecial_nf_, sel, store_,
                                         wide_, any_force_, any_links_, true, stream_));
    }
    bool first = true;
    for (int s = 0; s < max_stages_; s++) {
        // the first level's force blocks come last in its list
        const int nb = stage_nblocks_[s] - (s == 0 && !forces_ ? nforce_ : 0);
        if (nb <= 0) continue;
        CK(launch::stage_batch(d_stage_lists_[s], stage_counts_[s], d_stage_blocks_[s], nb, store_, sel, d_force_,
                               first, nodes_ < (1LL << 20), stream_));
        first = false;
    }
    if (forces_ && nforce_ && max_stages_ == 0) CK(launch::force_reduce(d_force_, nforce_, true, stream_));
    if (nrec_) {
        const int psize = store_ == STORE_F64 ? (int)sizeof(StepParams) : (int)sizeof(FastStepParams);
        CK(launch::record(d_rec_, nrec_, store_, nullptr, (const char *)d_sp_, psize, sel, true,
                          stream_));
    }
    return true;
}

bool Batch::capture_pair() {
    if (pair_exec_) return true;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    const bool okk = launch_batched(0) && launch_batched(1);
    const cudaError_t e = cudaStreamEndCapture(stream_, &g);
    if (!okk) {
        if (g) cudaGraphDestroy(g);
        return false;
    }
    CK(e);
    const cudaError_t e2 = cudaGraphInstantiate(&pair_exec_, g, 0);
    cudaGraphDestroy(g);
    CK(e2);
    return true;
}

bool Batch::run(int nsteps) {
    if (!ok_) return false;
    if (nsteps <= 0) return true;
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    bool okk = true;
    for (Solver *c : cases_) {
        okk = okk && check_cuda(cudaEventRecord(ev, c->stream()), "event") &&
              check_cuda(cudaStreamWaitEvent(stream_, ev, 0), "event");
    }
    for (Solver *c : cases_) okk = okk && c->begin_steps(stream_);
    const int mid = nsteps - 1;
    if (okk && mid > 0) {
        // Parameters of both ping-pong directions from each case's current state,
        // in host vectors that outlive the copies (the previous run's copies are
        // waited for before the vectors are refilled).
        const int nc = (int)cases_.size();
        if (params_ev_) okk = okk && check_cuda(cudaEventSynchronize(params_ev_), "event");
        std::vector<StepParams> &sp = h_sp_;
        std::vector<FastStepParams> &fsp = h_fsp_;
        std::vector<FinishParams> &fin = h_fin_;
        std::vector<std::vector<StageParams>> &lists = h_lists_;
        sp.assign(2 * nc, StepParams());
        fsp.assign(store_ == STORE_F64 ? 0 : 2 * nc, FastStepParams());
        fin.assign(2 * nc, FinishParams());
        lists.assign(max_stages_, std::vector<StageParams>());
        // The wall force of the batched steps is needed only by cases that
        // record it every step (force history): the run's last step, which
        // gives lbm_gpu_forces its value, is each case's own. Without a
        // history the batched steps store no force partials and reduce none
        // (measured on 64 liner ducts: see launch_batched).
        bool forces = false;
        for (Solver *c : cases_) forces = forces || c->hist_cap() > 0;
        if (forces != forces_ && pair_exec_) {
            cudaGraphExecDestroy(pair_exec_);
            pair_exec_ = nullptr;
        }
        forces_ = forces;
        for (int c = 0; c < nc; c++) {
            Solver *s = cases_[c];
            const int cur = s->current(), par = s->parity();
            sp[2 * c] = s->step_params(cur, 1 - cur, false, par);
            sp[2 * c + 1] = s->step_params(1 - cur, cur, false, par ^ 1);
            if (!forces) sp[2 * c].mem_partials = sp[2 * c + 1].mem_partials = nullptr;
            if (!fsp.empty()) {
                fsp[2 * c] = s->fast_params(sp[2 * c]);
                fsp[2 * c + 1] = s->fast_params(sp[2 * c + 1]);
            }
            fin[2 * c] = s->finish_params(1 - cur, false, par);
            fin[2 * c + 1] = s->finish_params(cur, false, par ^ 1);
            for (size_t l = 0; l < s->stage_groups().size(); l++)
                for (int k : s->stage_groups()[l]) {
                    lists[l].push_back(s->stage_params(s->stages()[k], cur, par));
                    lists[l].back().fin = d_fin_ + 2 * c;
                    lists[l].push_back(s->stage_params(s->stages()[k], 1 - cur, par ^ 1));
                    lists[l].back().fin = d_fin_ + 2 * c + 1;
                }
        }
        if (store_ == STORE_F64)
            okk = okk && check_cuda(cudaMemcpyAsync(d_sp_, sp.data(), sp.size() * sizeof(StepParams), cudaMemcpyHostToDevice, stream_), "H2D");
        else
            okk = okk && check_cuda(cudaMemcpyAsync(d_sp_, fsp.data(), fsp.size() * sizeof(FastStepParams), cudaMemcpyHostToDevice, stream_), "H2D");
        okk = okk && check_cuda(cudaMemcpyAsync(d_fin_, fin.data(), fin.size() * sizeof(FinishParams), cudaMemcpyHostToDevice, stream_), "H2D");
        for (int k = 0; k < max_stages_ && okk; k++)
            okk = check_cuda(cudaMemcpyAsync(d_stage_lists_[k], lists[k].data(), lists[k].size() * sizeof(StageParams), cudaMemcpyHostToDevice, stream_), "H2D");
        if (!params_ev_) okk = okk && check_cuda(cudaEventCreateWithFlags(&params_ev_, cudaEventDisableTiming), "event");
        okk = okk && check_cuda(cudaEventRecord(params_ev_, stream_), "event");
        int pairs = mid / 2;
        // Tuning takes its trial windows from the step pairs of this run.
        if (okk && tune_mode_ && !tuned_ && pairs >= 1 + 2 * kNTileCand) {
            const int used = tune_online(pairs);
            okk = used >= 0;
            pairs -= std::max(used, 0);
        }
        if (okk && pairs > 0) okk = capture_pair();
        for (; okk && pairs > 0; pairs--) okk = check_cuda(cudaGraphLaunch(pair_exec_, stream_), "graph");
        if (okk && (mid & 1)) okk = launch_batched(0);
        for (Solver *c : cases_) {
            c->advance(mid);
            c->add_steps(mid);
        }
    }
    for (Solver *c : cases_) {
        okk = okk && c->end_steps(stream_);
        c->add_steps(1);
    }
    okk = okk && check_cuda(cudaEventRecord(ev, stream_), "event");
    for (Solver *c : cases_) okk = okk && check_cuda(cudaStreamWaitEvent(c->stream(), ev, 0), "event");
    cudaEventDestroy(ev);
    return okk;
}

}  // namespace lbm
