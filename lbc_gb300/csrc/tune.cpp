// tune.cpp -- launch-shape autotuner support (see tune.h).
#include "tune.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <sstream>
#include <tuple>

#include "engine.h"

namespace lbm {

namespace {

struct Entry {
    int a, b;
    double us;
};

std::mutex g_mu;
std::map<std::string, Entry> g_table;
bool g_loaded = false;

const char *cache_path() {
    const char *p = std::getenv("LBM_GPU_TUNE_CACHE");
    return (p && *p) ? p : nullptr;
}

void load_locked() {
    if (g_loaded) return;
    g_loaded = true;
    const char *path = cache_path();
    if (!path) return;
    FILE *f = std::fopen(path, "r");
    if (!f) return;
    char line[512];
    while (std::fgets(line, sizeof line, f)) {
        std::istringstream is(line);
        std::string key;
        Entry e;
        if (is >> key >> e.a >> e.b >> e.us) g_table[key] = e;
    }
    std::fclose(f);
}

}  // namespace

std::string device_tag() {
    int dev = 0, maj = 0, min = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maj, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&min, cudaDevAttrComputeCapabilityMinor, dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return "sm" + std::to_string(maj) + std::to_string(min) + "x" + std::to_string(nsm);
}

bool tune_lookup(const std::string &key, int &a, int &b) {
    std::lock_guard<std::mutex> lk(g_mu);
    load_locked();
    auto it = g_table.find(key);
    if (it == g_table.end()) return false;
    a = it->second.a;
    b = it->second.b;
    return true;
}

void tune_store(const std::string &key, int a, int b, double us) {
    std::lock_guard<std::mutex> lk(g_mu);
    load_locked();
    g_table[key] = Entry{a, b, us};
    const char *path = cache_path();
    if (!path) return;
    FILE *f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%s %d %d %.3f\n", key.c_str(), a, b, us);
    std::fclose(f);
}

void tune_clear() {
    std::lock_guard<std::mutex> lk(g_mu);
    g_table.clear();
    g_loaded = true;  // do not re-read the file after an explicit clear
}

int tune_default_mode() {
    const char *v = std::getenv("LBM_GPU_AUTOTUNE");
    return (v && std::atoi(v) != 0) ? 1 : 0;
}

WindowTimer::WindowTimer(int nwindows) : ev_(nwindows + 1, nullptr), ms_(nwindows, 0.f) {
    for (cudaEvent_t &e : ev_)
        if (!check_cuda(cudaEventCreate(&e), "cudaEventCreate")) return;
    ok_ = true;
}

WindowTimer::~WindowTimer() {
    for (cudaEvent_t e : ev_)
        if (e) cudaEventDestroy(e);
}

bool WindowTimer::mark(int k, cudaStream_t s) { return check_cuda(cudaEventRecord(ev_[k], s), "cudaEventRecord"); }

bool WindowTimer::wait() {
    if (!check_cuda(cudaEventSynchronize(ev_.back()), "cudaEventSynchronize")) return false;
    for (size_t k = 0; k + 1 < ev_.size(); k++)
        if (!check_cuda(cudaEventElapsedTime(&ms_[k], ev_[k], ev_[k + 1]), "cudaEventElapsedTime")) return false;
    return true;
}

float WindowTimer::elapsed(int k) const { return ms_[k]; }

int window_steps(float est_ms, float target_ms, int lo, int hi) {
    if (!(est_ms > 0.f)) return lo;
    const int k = (int)std::ceil(target_ms / est_ms);
    return k < lo ? lo : (k > hi ? hi : k);
}

}  // namespace lbm
