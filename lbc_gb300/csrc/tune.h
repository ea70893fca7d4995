// tune.h -- launch-shape autotuner: cache of tuned shapes and the timing of
// trial windows (internal header).
//
// The fused step's populations do not depend on the thread-block shape of the
// single-case kernel or on the tile shape of the batched kernel, and the force
// partials are per 32-node row segment, so the momentum-exchange force does
// not either. The tuner therefore times candidate shapes on the first steps of
// a real run (each trial step is one of the steps asked for) and keeps the
// fastest for the rest: no scratch memory, no extra steps, no effect on any
// result.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace lbm {

// "sm<major><minor>x<SMs>" of the current device.
std::string device_tag();

// Process-wide table key -> (a, b, microseconds per step). When the
// environment variable LBM_GPU_TUNE_CACHE names a file, the table is read from
// it on first use and each new entry is appended to it (one line per entry:
// key a b us).
bool tune_lookup(const std::string &key, int &a, int &b);
void tune_store(const std::string &key, int a, int b, double us);
void tune_clear();

// 1 when LBM_GPU_AUTOTUNE is set to a nonzero integer: new solvers and
// batches then tune on their first long enough run.
int tune_default_mode();

// Events around consecutive trial windows on one stream: mark(k) before
// window k, mark(n) after the last; elapsed(k) = milliseconds of window k.
class WindowTimer {
  public:
    explicit WindowTimer(int nwindows);
    ~WindowTimer();
    bool ok() const { return ok_; }
    bool mark(int k, cudaStream_t s);
    bool wait();
    float elapsed(int k) const;

  private:
    std::vector<cudaEvent_t> ev_;
    std::vector<float> ms_;
    bool ok_ = false;
};

// Number of steps per trial window: enough for about `target_ms` of work at
// `est_ms` per step, in [lo, hi].
int window_steps(float est_ms, float target_ms, int lo, int hi);

}  // namespace lbm
