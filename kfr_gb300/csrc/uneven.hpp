// Many signals of uneven lengths, stored back to back, transformed by one persistent launch.
//
// The reference has no batch API: a caller loops over dft_plan<T>::execute, one plan per length
// (include/kfr/dft/fft.hpp:265-272).  Here one persistent kernel drains a device work queue of tiles:
//   DIRECT  up to `spc` whole signals of one length whose transform fits one CTA;
//   BLUE1   the same for a length with a large prime factor, through a one-CTA Bluestein convolution;
//   COL/ROW a tile of the column or row pass of a four-step transform of a longer signal (N = n1 * n2).  A
//           Bluestein transform whose convolution is too long for one CTA runs as two four-step transforms,
//           with the chirp, the kernel spectrum and the final chirp fused into their first load and last
//           stores.
// The queue lists every tile of a stage after all tiles of the stage before it; a tile that depends on an
// earlier stage of its signal waits (bounded, with an error flag) for that stage's tile counter, which the
// earlier tiles, all already dequeued by resident CTAs, raise when they finish.  The whole launch is captured
// once per (in, out, direction) as a CUDA graph and replayed.  A small autotuner times the candidate radix
// orders and tile shapes of each one-CTA length on the device when the plan is built and keeps the fastest
// in a process-wide cache keyed by length.
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "plan.hpp"

namespace kfr_gpu
{

// block FFT shape run inside a tile
struct uneven_fft
{
    fft_desc d;
    const void* tw;
    int m, ts, stride;
    fast_div div_m;
};

enum uneven_mode
{
    UM_DIRECT = 0,
    UM_BLUE1  = 1,
    UM_COL    = 2,
    UM_ROW    = 3,
};

// one job: a length class (DIRECT / BLUE1, over the signals its items list) or one stage of one long signal
struct uneven_job
{
    int mode;
    int fft;            // index of the block FFT shape
    int n;              // DIRECT / BLUE1: signal length; COL / ROW: n1 / n2 of the split
    int n1, n2;         // COL / ROW
    int src, dst;       // buffers: 0 = in, 1 = out, 2 = scratch
    long long src_off;  // COL / ROW: element offset of the signal (or its scratch) in src / dst
    long long dst_off;
    int pre;            // COL: 0 plain, 1 times chirp with the signal (length nvalid) zero padded
    int post;           // ROW: 0 plain, 1 conj(v * bhat), 2 conj(v) * chirp for k < nvalid
    int first, last;    // conjugate on load (first stage) / on store (last stage) for the inverse
    long long nvalid;
    const void* chirp;
    const void* bhat;
    const void* twA;    // four-step twiddle W_N^m = twA[m >> lbits] * twB[m & mask]
    const void* twB;
    int lbits;
    int wait, need;     // counter to wait for (-1: none) and its required value
    int done;           // counter raised when an item of this job finishes (-1: none)
};

struct uneven_item
{
    int job;
    int first; // DIRECT / BLUE1: index of the first signal in the offset list; COL / ROW: first column / row
    int count; // signals (DIRECT / BLUE1) or columns / rows (COL / ROW)
};

// Threads of the persistent kernel (one CTA per SM; block FFTs of up to 8192 points, 16 values per thread).
constexpr int kUnevenThreads = 512;
// Most signals or columns one work item carries.
constexpr int kUnevenMaxSpc = 256;

struct uneven_launch
{
    const uneven_fft* ffts;
    const uneven_job* jobs;
    const uneven_item* items;
    const long long* offsets;
    int nitems;
    int* queue;     // work counter
    int* counters;  // stage counters
    int* err;
    const void* in;
    void* out;
    void* scratch;
    int inverse;
    unsigned wait_spins; // polls (256 ns sleeps) before a stage wait gives up (kDefaultWaitSpins, launch.hpp)
    int stage_bias;      // added to every stage count waited for: 0, or 1 to make every such wait run out
};

cudaError_t launch_uneven_f32(const uneven_launch& a, int smem, int grid, cudaStream_t st);
int uneven_max_smem();

class uneven_plan
{
public:
    // lengths of the signals in storage order; autotune: time candidate radix orders and tiles per length
    uneven_plan(const std::vector<long long>& lengths, bool autotune);
    ~uneven_plan();
    // device pointers; enqueued on st (a captured graph is replayed after the first call with these pointers)
    void execute(void* out, const void* in, bool inverse, cudaStream_t st);
    // the plain form: one regular plan execution (and its launches) per signal
    void execute_per_signal(void* out, const void* in, bool inverse, cudaStream_t st);
    // raises if a tile gave up waiting for its dependencies (call after synchronising)
    void check_device_error() const;
    // failure-detection test: every tile that depends on an earlier stage waits for one more tile than that
    // stage has, so its wait runs out (after the wait limit) and the device error flag is set
    void set_unreachable_stage(bool on) { unreachable_ = on; }
    long long total() const { return total_; }
    std::string describe() const;

private:
    struct shape
    {
        block_program<float> prog;
        int ts = 1;
    };
    std::vector<long long> lengths_, offsets_;
    long long total_ = 0;
    std::vector<std::unique_ptr<shape>> shapes_;
    std::map<std::pair<long long, int>, int> shape_of_; // (m, threads cap) -> shape
    std::vector<std::unique_ptr<dbuf>> tables_;         // chirps, spectra and four-step twiddles
    dbuf dffts_, djobs_, ditems_, doffsets_, dqueue_, dcounters_, derr_, scratch_;
    int nitems_ = 0, ncounters_ = 0, smem_ = 0, grid_ = 0;
    int n_direct_ = 0, n_blue1_ = 0, n_fourstep_ = 0, n_blue_fs_ = 0;
    std::map<long long, std::unique_ptr<complex_engine<float>>> engines_; // plain form only
    dbuf plain_scratch_;
    cudaStream_t cap_ = nullptr;
    cudaGraphExec_t gexec_ = nullptr;
    const void* gin_ = nullptr;
    void* gout_      = nullptr;
    bool ginv_       = false;
    bool unreachable_ = false;
    unsigned gspins_  = 0; // wait settings the captured graph was built with
    bool gunreach_    = false;

    int get_shape(long long m, int max_ts, const std::vector<int>* order = nullptr);
    void enqueue(void* out, const void* in, bool inverse, cudaStream_t st);
};

} // namespace kfr_gpu
