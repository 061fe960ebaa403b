// Scratch buffers of the entry points that only enqueue work on the caller's
// stream (the *_dev calls, libconv_cg_apply).  Such a call returns while its
// kernels still use their scratch (dot partials, line exponents, partial
// sums), so two calls on different streams must never share one buffer set.
//
// StreamPool hands one entry (a set of device buffers) to one call at a
// time.  acquire() prefers the entry last used on the same stream (stream
// order already separates the two calls), then an idle entry, then a new one
// (up to kPoolMax), and only when every entry is busy on another stream the
// oldest one (a slow path that only calls in flight on more than kPoolMax
// streams at once reach); the call's stream then waits on that entry's
// completion event
// before any of its own work, so the worst case serialises the calls, never
// mixes their data.  release() records the event after the call's work.  A
// buffer grows only after its previous user finished (event synchronised),
// before the new call enqueued anything.  An entry leased while the stream
// is being captured into a CUDA graph belongs to that graph from then on and
// is never handed out again.  The owner of the pool serialises acquire() /
// release() (its library lock).
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace lcg {

constexpr int kPoolBufs = 4;
constexpr size_t kPoolMax = 16;

struct PoolEntry {
    void *p[kPoolBufs] = {nullptr, nullptr, nullptr, nullptr};
    size_t cap[kPoolBufs] = {0, 0, 0, 0};
    cudaEvent_t done = nullptr;
    cudaStream_t last = nullptr;
    bool used = false;       // done has been recorded at least once
    bool captured = false;   // owned by a captured graph
    unsigned long long stamp = 0;
};

class StreamPool {
  public:
    // Lease an entry whose buffer k holds at least bytes[k] (k < nb) for work
    // enqueued on st.  On error nothing is leased.
    cudaError_t acquire(cudaStream_t st, const size_t *bytes, int nb, PoolEntry *&out) {
        out = nullptr;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaError_t e = cudaStreamIsCapturing(st, &cs);
        if (e != cudaSuccess) return e;
        const bool capturing = cs != cudaStreamCaptureStatusNone;
        PoolEntry *pick = nullptr;
        if (!capturing) {
            // the stream's own entry (not for the per-thread default stream,
            // whose one handle names a different stream in every thread)
            if (st != cudaStreamPerThread)
                for (PoolEntry *x : entries_)
                    if (!x->captured && x->used && x->last == st && (!pick || x->stamp > pick->stamp))
                        pick = x;
            for (size_t i = 0; !pick && i < entries_.size(); ++i) {   // an idle one
                PoolEntry *x = entries_[i];
                if (x->captured) continue;
                if (!x->used) { pick = x; break; }
                const cudaError_t q = cudaEventQuery(x->done);
                if (q == cudaSuccess) pick = x;
                else if (q != cudaErrorNotReady) return q;
            }
            if (!pick && entries_.size() >= kPoolMax)                 // all busy: the oldest
                for (PoolEntry *x : entries_)
                    if (!x->captured && (!pick || x->stamp < pick->stamp)) pick = x;
        }
        if (!pick) {
            pick = new PoolEntry();
            e = cudaEventCreateWithFlags(&pick->done, cudaEventDisableTiming);
            if (e != cudaSuccess) { delete pick; return e; }
            entries_.push_back(pick);
        }
        for (int k = 0; k < nb && k < kPoolBufs; ++k) {
            if (pick->cap[k] >= bytes[k]) continue;
            if (pick->used && (e = cudaEventSynchronize(pick->done)) != cudaSuccess) return e;
            if (pick->p[k]) cudaFree(pick->p[k]);
            pick->p[k] = nullptr;
            pick->cap[k] = 0;
            const size_t want = bytes[k] < 256 ? 256 : bytes[k];
            if ((e = cudaMalloc(&pick->p[k], want)) != cudaSuccess) {
                pick->p[k] = nullptr;
                return e;
            }
            pick->cap[k] = want;
        }
        // after the entry's previous user (a no-op when that was this stream)
        if (pick->used && (e = cudaStreamWaitEvent(st, pick->done, 0)) != cudaSuccess) return e;
        if (capturing) pick->captured = true;
        out = pick;
        return cudaSuccess;
    }

    // The call has enqueued all its work on st.
    cudaError_t release(PoolEntry *x, cudaStream_t st) {
        if (!x || x->captured) return cudaSuccess;
        const cudaError_t e = cudaEventRecord(x->done, st);
        if (e != cudaSuccess) return e;
        x->used = true;
        x->last = st;
        x->stamp = ++clock_;
        return cudaSuccess;
    }

    size_t size() const { return entries_.size(); }

  private:
    std::vector<PoolEntry *> entries_;
    unsigned long long clock_ = 0;
};

}  // namespace lcg
