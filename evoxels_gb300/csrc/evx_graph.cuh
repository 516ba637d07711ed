// Repeated multi-step calls replayed as CUDA graphs.
//
// A plan's forward and adjoint loops launch several kernels and cuFFT
// executions per step; on small grids the gaps between those dependent
// launches are a large part of the step.  A GraphCache keys each call by
// everything its launches bake in (pointers, step count, parameters) and
//   - runs the first call with a key eagerly,
//   - captures the second call with the same key on a private non-blocking
//     stream (thread-local capture mode), instantiates it and launches the
//     graph on the caller's stream,
//   - launches that graph for every later call with the key.
// A call that cannot be captured (a capture error, a failed instantiation)
// runs eagerly from then on.  Calls made while the caller's stream is itself
// being captured, or while kernel timing is on, always run eagerly.  A change
// of kernel choice (the stencil tile shape) drops every cached graph.  The
// graphs hold the same kernels with the same arguments as the eager path, so
// results are bit-identical.  The launch counter counts a replayed graph's
// kernels once per replay.
#pragma once

#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "evx_prof.cuh"

namespace evx {

bool graphs_enabled();                       // evx_set_graphs; off while kernel timing is on
unsigned long long launch_counter();
void uncount_launch(unsigned long long n);   // undo the counts of a capture (nothing ran)
unsigned long long config_epoch();           // bumped by every change of kernel choice
void bump_config_epoch();

using GraphKey = std::vector<uint64_t>;

inline uint64_t key_p(const void* p) { return (uint64_t)reinterpret_cast<uintptr_t>(p); }
inline uint64_t key_f(float v) {
    uint32_t u;
    std::memcpy(&u, &v, sizeof(u));
    return u;
}

class GraphCache {
  public:
    static constexpr int CAP = 4;   // keys kept per cache (least recently used evicted)

    GraphCache() = default;
    GraphCache(const GraphCache&) = delete;
    GraphCache& operator=(const GraphCache&) = delete;
    ~GraphCache() {
        // an executable graph still running is freed when its launch completes
        for (auto& e : ents_)
            if (e.exec) cudaGraphExecDestroy(e.exec);
        if (cap_) cudaStreamDestroy(cap_);
    }

    // body(stream) issues the call's work on the given stream and returns an
    // evx status.
    template <class F>
    int run(const GraphKey& key, cudaStream_t st, F&& body) {
        if (!graphs_enabled()) return body(st);
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
            cudaGetLastError();
            return body(st);
        }
        if (cs != cudaStreamCaptureStatusNone) return body(st);
        std::lock_guard<std::mutex> lk(mu_);
        const unsigned long long ep = config_epoch();
        if (ep != epoch_) {
            for (auto& x : ents_)
                if (x.exec) cudaGraphExecDestroy(x.exec);
            ents_.clear();
            epoch_ = ep;
        }
        ++tick_;
        Ent* e = find(key);
        if (!e) {   // first sighting
            insert(key);
            return body(st);
        }
        e->used = tick_;
        if (e->never) return body(st);
        if (!e->exec) {
            capture(*e, body);
            if (!e->exec) return body(st);
        }
        const int rc = check_cuda(cudaGraphLaunch(e->exec, st), "cudaGraphLaunch");
        if (!rc) count_launch((unsigned)e->launches);
        return rc;
    }

  private:
    struct Ent {
        GraphKey key;
        cudaGraphExec_t exec = nullptr;
        unsigned long long launches = 0;
        unsigned long long used = 0;
        bool never = false;
    };

    Ent* find(const GraphKey& key) {
        for (auto& e : ents_)
            if (e.key == key) return &e;
        return nullptr;
    }

    void insert(const GraphKey& key) {
        if ((int)ents_.size() >= CAP) {
            size_t lru = 0;
            for (size_t i = 1; i < ents_.size(); ++i)
                if (ents_[i].used < ents_[lru].used) lru = i;
            if (ents_[lru].exec) cudaGraphExecDestroy(ents_[lru].exec);
            ents_.erase(ents_.begin() + (long)lru);
        }
        Ent e;
        e.key = key;
        e.used = tick_;
        ents_.push_back(std::move(e));
    }

    template <class F>
    void capture(Ent& e, F& body) {
        e.never = true;   // unless everything below succeeds
        if (!cap_ && cudaStreamCreateWithFlags(&cap_, cudaStreamNonBlocking) != cudaSuccess) {
            cap_ = nullptr;
            cudaGetLastError();
            return;
        }
        if (cudaStreamBeginCapture(cap_, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        const unsigned long long c0 = launch_counter();
        const int rc = body(cap_);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(cap_, &g);
        const unsigned long long n = launch_counter() - c0;
        uncount_launch(n);
        if (rc || ce != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return;
        }
        cudaGraphExec_t x = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&x, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess || !x) {
            cudaGetLastError();
            return;
        }
        e.exec = x;
        e.launches = n;
        e.never = false;
    }

    std::mutex mu_;
    std::vector<Ent> ents_;
    unsigned long long epoch_ = 0;
    cudaStream_t cap_ = nullptr;
    unsigned long long tick_ = 0;
};

}  // namespace evx
