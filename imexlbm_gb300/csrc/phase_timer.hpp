// Device-time accounting of a lattice's kernel launches by phase, for the
// per-phase profile report (the reference's lbmprof, src/profile.hpp /
// src/profile.cpp, which times host-side phases with MPI_Wtime around
// fences).  Here each phase's launches are bracketed by CUDA events on the
// launching stream, so timing adds no synchronisation to the step; the
// events are read back - and the per-launch times folded into calls /
// total / min / max - when the report is read, or when many are pending.
// Launches queued while the stream is being captured into a graph are not
// timed (events cannot be timed inside a graph).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "imexlbm.h"

namespace imex {

class PhaseTimer {
public:
    ~PhaseTimer() { release(); }

    bool enabled() const { return on_; }

    void enable(bool on)
    {
        if (!on) collect();
        on_ = on;
    }

    // Start timing one launch of `phase` on stream s; returns a token for
    // stop() (-1: not timed).
    int start(int phase, cudaStream_t s)
    {
        if (!on_) return -1;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
            cudaGetLastError();
            return -1;
        }
        if (pending_.size() >= kMaxPending) collect();
        Pair p{phase, take(), take()};
        if (!p.a || !p.b || cudaEventRecord(p.a, s) != cudaSuccess) {
            cudaGetLastError();
            give(p.a);
            give(p.b);
            return -1;
        }
        pending_.push_back(p);
        return (int)pending_.size() - 1;
    }

    void stop(int token, cudaStream_t s)
    {
        if (token < 0 || token >= (int)pending_.size()) return;
        if (cudaEventRecord(pending_[token].b, s) != cudaSuccess) {
            cudaGetLastError();
            pending_[token].phase = -1;  // dropped at collection
        }
    }

    // Fold every pending launch into the statistics (waits for them).
    void collect()
    {
        for (Pair& p : pending_) {
            float ms = 0.f;
            if (p.phase >= 0 && cudaEventSynchronize(p.b) == cudaSuccess &&
                cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
                imex_phase_stats& st = stats_[p.phase];
                if (st.calls == 0 || ms < st.min_ms) st.min_ms = ms;
                if (st.calls == 0 || ms > st.max_ms) st.max_ms = ms;
                st.total_ms += ms;
                ++st.calls;
            }
            cudaGetLastError();
            give(p.a);
            give(p.b);
        }
        pending_.clear();
    }

    void read(imex_phase_stats out[IMEX_NPHASE], bool reset)
    {
        collect();
        for (int q = 0; q < IMEX_NPHASE; ++q) {
            out[q] = stats_[q];
            if (reset) stats_[q] = imex_phase_stats{};
        }
    }

    void release()
    {
        collect();
        for (cudaEvent_t e : free_) cudaEventDestroy(e);
        free_.clear();
    }

private:
    struct Pair {
        int phase;
        cudaEvent_t a, b;
    };
    static constexpr size_t kMaxPending = 512;

    cudaEvent_t take()
    {
        if (!free_.empty()) {
            cudaEvent_t e = free_.back();
            free_.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        return e;
    }
    void give(cudaEvent_t e)
    {
        if (e) free_.push_back(e);
    }

    bool on_ = false;
    std::vector<Pair> pending_;
    std::vector<cudaEvent_t> free_;
    imex_phase_stats stats_[IMEX_NPHASE] = {};
};

// Times one launch for the lifetime of the object.
struct PhaseScope {
    PhaseTimer& t;
    cudaStream_t s;
    int token;
    PhaseScope(PhaseTimer& timer, int phase, cudaStream_t stream) : t(timer), s(stream), token(timer.start(phase, stream)) {}
    ~PhaseScope() { t.stop(token, s); }
};

}  // namespace imex
