// io.cu -- population checkpoints and device-packed VTK output of a Solver.
//
// Checkpoint file (little-endian host order; the file is for this library on
// this machine type, not an exchange format):
//   "LBMGPUCP" | u32 version | i32 Nx, Ny, pitch, storage, cur, parity,
//   fields_are_moments, nslots, nstages, hist_cap | i64 steps_done
//   then blobs (u64 byte count, bytes): both population buffers (device SoA
//   planes as stored), rho, u, v (FP64), the two band-moment buffers, per
//   stage its val1, val2 and impedance-wall state, the last force, and the
//   force-history ring with its counter.
// The geometry tables are not stored: they are rebuilt from the case when the
// loading solver is created, and the header and blob sizes must match it.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "engine.h"

namespace lbm {

#define CK(call)                                \
    do {                                        \
        if (!check_cuda((call), #call)) return false; \
    } while (0)

namespace {

const char kMagic[8] = {'L', 'B', 'M', 'G', 'P', 'U', 'C', 'P'};
constexpr uint32_t kVersion = 1;

struct Header {
    char magic[8];
    uint32_t version;
    int32_t Nx, Ny, pitch, store, cur, parity, fields_are_moments, nslots, nstages, hist_cap;
    int64_t steps_done;
};

bool put_blob(FILE *f, const void *dev, size_t bytes, std::vector<unsigned char> &tmp) {
    const uint64_t n = bytes;
    if (fwrite(&n, sizeof n, 1, f) != 1) return false;
    if (!bytes) return true;
    tmp.resize(bytes);
    if (!check_cuda(cudaMemcpy(tmp.data(), dev, bytes, cudaMemcpyDeviceToHost), "checkpoint D2H")) return false;
    return fwrite(tmp.data(), 1, bytes, f) == bytes;
}

bool get_blob(FILE *f, void *dev, size_t bytes, std::vector<unsigned char> &tmp, const char *what) {
    uint64_t n = 0;
    if (fread(&n, sizeof n, 1, f) != 1) {
        set_error(std::string("checkpoint: truncated before ") + what);
        return false;
    }
    if (n != bytes) {
        set_error(std::string("checkpoint: ") + what + " has " + std::to_string(n) + " bytes, this solver " +
                  std::to_string(bytes));
        return false;
    }
    if (!bytes) return true;
    tmp.resize(bytes);
    if (fread(tmp.data(), 1, bytes, f) != bytes) {
        set_error(std::string("checkpoint: truncated in ") + what);
        return false;
    }
    return check_cuda(cudaMemcpy(dev, tmp.data(), bytes, cudaMemcpyHostToDevice), "checkpoint H2D");
}

// Big-endian IEEE single of (float)(x * c), as lbc's writer stores it.
__device__ __forceinline__ unsigned int be32(double x, double c) {
    const float v = __double2float_rn(__dmul_rn(x, c));
    return __byte_perm(__float_as_uint(v), 0, 0x0123);
}

// Payload of write_vtk_binary_2D (src/utils/write_vtk_binary_2D.c:46-78):
// N velocity 3-vectors (u, v, 0), then N densities, big-endian FP32.
__global__ void k_pack_vtk(int N, const double *__restrict__ rho, const double *__restrict__ u,
                           const double *__restrict__ v, double cu, double crho,
                           unsigned int *__restrict__ out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    out[3 * (size_t)n] = be32(u[n], cu);
    out[3 * (size_t)n + 1] = be32(v[n], cu);
    out[3 * (size_t)n + 2] = 0u;  // +0.0f is all zero bits in either byte order
    out[3 * (size_t)N + n] = be32(rho[n], crho);
}

}  // namespace

bool Solver::checkpoint_save(const char *path) {
    if (!path) {
        set_error("checkpoint: null path");
        return false;
    }
    CK(cudaStreamSynchronize(stream_));
    FILE *f = fopen(path, "wb");
    if (!f) {
        set_error(std::string("checkpoint: cannot open ") + path + " for writing");
        return false;
    }
    Header h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.Nx = d_.Nx; h.Ny = d_.Ny; h.pitch = pitch_; h.store = d_.store;
    h.cur = cur_; h.parity = parity_; h.fields_are_moments = fields_are_moments_ ? 1 : 0;
    h.nslots = nslots_; h.nstages = (int)stages_.size(); h.hist_cap = hist_cap_;
    h.steps_done = steps_done_;
    const size_t N = (size_t)d_.Nx * d_.Ny, pop = (size_t)plane_ * 9 * esize_;
    std::vector<unsigned char> tmp;
    bool okk = fwrite(&h, sizeof h, 1, f) == 1 && put_blob(f, buf_[0], pop, tmp) && put_blob(f, buf_[1], pop, tmp) &&
               put_blob(f, d_rho_, N * 8, tmp) && put_blob(f, d_ux_, N * 8, tmp) && put_blob(f, d_uy_, N * 8, tmp);
    for (int b = 0; b < 2 && okk; b++) okk = put_blob(f, d_bandm_[b], nslots_ ? (size_t)nslots_ * 3 * 8 : 0, tmp);
    for (const Stage &st : stages_) {
        if (!okk) break;
        const size_t vb = st.d_val1 ? (size_t)st.along * 8 : 0;
        const size_t ib = st.d_imp ? imp_doubles(st.imp_nf, st.along) * 8 : 0;
        okk = put_blob(f, st.d_val1, vb, tmp) && put_blob(f, st.d_val2, vb, tmp) && put_blob(f, st.d_imp, ib, tmp);
    }
    okk = okk && put_blob(f, d_mem_out_, d_mem_out_ ? 16 : 0, tmp) &&
          put_blob(f, d_hist_, d_hist_ ? (size_t)hist_cap_ * 16 : 0, tmp) &&
          put_blob(f, hist_count_ptr_, hist_count_ptr_ ? 8 : 0, tmp);
    if (fclose(f) != 0) okk = false;
    if (!okk && std::string(last_error()).empty()) set_error(std::string("checkpoint: write failed: ") + path);
    return okk;
}

bool Solver::checkpoint_load(const char *path) {
    if (!path) {
        set_error("checkpoint: null path");
        return false;
    }
    FILE *f = fopen(path, "rb");
    if (!f) {
        set_error(std::string("checkpoint: cannot open ") + path);
        return false;
    }
    Header h;
    bool okk = fread(&h, sizeof h, 1, f) == 1;
    if (!okk || std::memcmp(h.magic, kMagic, 8) != 0 || h.version != kVersion) {
        fclose(f);
        set_error("checkpoint: not a checkpoint of this library (magic or version)");
        return false;
    }
    if (h.Nx != d_.Nx || h.Ny != d_.Ny || h.pitch != pitch_ || h.store != d_.store || h.nslots != nslots_ ||
        h.nstages != (int)stages_.size() || h.hist_cap != hist_cap_) {
        fclose(f);
        set_error("checkpoint: grid, storage, edge stages or force-history capacity differ from this solver");
        return false;
    }
    CK(cudaStreamSynchronize(stream_));
    const size_t N = (size_t)d_.Nx * d_.Ny, pop = (size_t)plane_ * 9 * esize_;
    std::vector<unsigned char> tmp;
    okk = get_blob(f, buf_[0], pop, tmp, "populations 0") && get_blob(f, buf_[1], pop, tmp, "populations 1") &&
          get_blob(f, d_rho_, N * 8, tmp, "rho") && get_blob(f, d_ux_, N * 8, tmp, "u") &&
          get_blob(f, d_uy_, N * 8, tmp, "v");
    for (int b = 0; b < 2 && okk; b++)
        okk = get_blob(f, d_bandm_[b], nslots_ ? (size_t)nslots_ * 3 * 8 : 0, tmp, "band moments");
    for (Stage &st : stages_) {
        if (!okk) break;
        const size_t vb = st.d_val1 ? (size_t)st.along * 8 : 0;
        const size_t ib = st.d_imp ? imp_doubles(st.imp_nf, st.along) * 8 : 0;
        okk = get_blob(f, st.d_val1, vb, tmp, "BC values") && get_blob(f, st.d_val2, vb, tmp, "BC values") &&
              get_blob(f, st.d_imp, ib, tmp, "impedance wall (set the same wall up before loading)");
    }
    okk = okk && get_blob(f, d_mem_out_, d_mem_out_ ? 16 : 0, tmp, "force") &&
          get_blob(f, d_hist_, d_hist_ ? (size_t)hist_cap_ * 16 : 0, tmp, "force history") &&
          get_blob(f, hist_count_ptr_, hist_count_ptr_ ? 8 : 0, tmp, "force history count");
    fclose(f);
    if (!okk) return false;
    cur_ = h.cur;
    parity_ = h.parity;
    fields_are_moments_ = h.fields_are_moments != 0;
    steps_done_ = h.steps_done;
    graph_valid_ = false;
    return true;
}

bool Solver::write_vtk(const char *path, double dx, double cu, double crho) {
    if (!path) {
        set_error("vtk: null path");
        return false;
    }
    if (!vtk_wait()) return false;  // one write in flight per solver
    const int Nx = d_.Nx, Ny = d_.Ny;
    const size_t N = (size_t)Nx * Ny, bytes = 16 * N;
    if (bytes != vtk_bytes_) {
        if (h_vtk_) cudaFreeHost(h_vtk_);
        h_vtk_ = nullptr;
        void *q = nullptr;
        if (!device_alloc(&q, bytes, stream_)) return false;
        allocs_.push_back(q);
        dev_bytes_ += bytes;
        d_vtk_ = (unsigned char *)q;
        CK(cudaMallocHost(&h_vtk_, bytes));
        vtk_bytes_ = bytes;
    }
    if (!vtk_ev_) CK(cudaEventCreateWithFlags(&vtk_ev_, cudaEventDisableTiming));
    // Pack and copy on the solver's stream: ordered after the step that wrote
    // the fields and before the next run overwrites them.
    k_pack_vtk<<<(unsigned)((N + 255) / 256), 256, 0, stream_>>>((int)N, d_rho_, d_ux_, d_uy_, cu, crho,
                                                                  (unsigned int *)d_vtk_);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h_vtk_, d_vtk_, bytes, cudaMemcpyDeviceToHost, stream_));
    CK(cudaEventRecord(vtk_ev_, stream_));
    const std::string file(path);
    vtk_ok_ = true;
    vtk_err_.clear();
    vtk_thread_ = new std::thread([this, file, Nx, Ny, dx, N] {
        if (cudaEventSynchronize(vtk_ev_) != cudaSuccess) {
            vtk_ok_ = false;
            vtk_err_ = "vtk: device copy failed";
            return;
        }
        FILE *fd = fopen(file.c_str(), "wb");
        if (!fd) {
            vtk_ok_ = false;
            vtk_err_ = "vtk: cannot open " + file;
            return;
        }
        // Header text as src/utils/write_vtk_binary_2D.c:46-62 writes it.
        fprintf(fd, "# vtk DataFile Version 3.0\n2D LBM output\nBINARY\nDATASET STRUCTURED_POINTS\n");
        fprintf(fd, "DIMENSIONS %d %d 1\n", Nx, Ny);
        fprintf(fd, "ORIGIN 0 0 0\n");
        fprintf(fd, "SPACING %f %f 1\n", dx, dx);
        fprintf(fd, "\nPOINT_DATA %d\n", Nx * Ny);
        fprintf(fd, "VECTORS velocity float\n");
        bool w = fwrite(h_vtk_, 1, 12 * N, fd) == 12 * N;
        fprintf(fd, "\nSCALARS density float 1\n");
        fprintf(fd, "LOOKUP_TABLE default\n");
        w = w && fwrite(h_vtk_ + 12 * N, 1, 4 * N, fd) == 4 * N;
        if (fclose(fd) != 0 || !w) {
            vtk_ok_ = false;
            vtk_err_ = "vtk: write failed: " + file;
        }
    });
    return true;
}

bool Solver::vtk_wait() {
    if (vtk_thread_) {
        vtk_thread_->join();
        delete vtk_thread_;
        vtk_thread_ = nullptr;
        if (!vtk_ok_) {
            set_error(vtk_err_);
            return false;
        }
    }
    return true;
}

}  // namespace lbm
