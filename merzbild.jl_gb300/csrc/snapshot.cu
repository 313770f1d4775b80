// Asynchronous read-back of cell properties and page-locked host memory.
//
// A time loop that reads the properties of every step (the reference's loops
// call compute_props! and read phys_props each output step) would otherwise
// stop the device at every read.  mz_props_snapshot copies the set into one
// of two device snapshot buffers on the context's stream (a few microseconds
// of device copies), then a side stream copies the snapshot to host memory
// while the next steps run.  A snapshot buffer is refilled only after its
// previous host copy finished (a device-side wait, no host block).
#include "mz_host.h"

struct PropsSnapshot {
    cudaStream_t side = nullptr;
    double* buf[2] = {nullptr, nullptr};
    cudaEvent_t ready[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    bool used[2] = {false, false};
    size_t doubles = 0;
};

void free_props_snapshot(mz_props* p)
{
    PropsSnapshot* s = static_cast<PropsSnapshot*>(p->snapshot);
    if (!s) return;
    if (s->side) cudaStreamSynchronize(s->side);
    for (int k = 0; k < 2; ++k) {
        if (s->buf[k]) cudaFree(s->buf[k]);
        if (s->ready[k]) cudaEventDestroy(s->ready[k]);
        if (s->done[k]) cudaEventDestroy(s->done[k]);
    }
    if (s->side) cudaStreamDestroy(s->side);
    delete s;
    p->snapshot = nullptr;
}

extern "C" {

int mz_props_snapshot(mz_props* p, int32_t slot, double* dst)
{
    API_TRY
    MZ_REQUIRE(p && dst && (slot == 0 || slot == 1), "mz_props_snapshot: bad argument");
    mz_domain* d = p->dom;
    mz_ctx* c = d->ctx;
    MZ_CK(cudaSetDevice(c->device));
    const size_t m = (size_t)d->n_cells * d->ns;
    PropsSnapshot* s = static_cast<PropsSnapshot*>(p->snapshot);
    if (!s) {
        s = new PropsSnapshot();
        p->snapshot = s;
        s->doubles = 6 * m;
        MZ_CK(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            MZ_CK(cudaMalloc(&s->buf[k], s->doubles * sizeof(double)));
            MZ_CK(cudaEventCreateWithFlags(&s->ready[k], cudaEventDisableTiming));
            MZ_CK(cudaEventCreateWithFlags(&s->done[k], cudaEventDisableTiming));
        }
    }
    // the slot's previous host copy must have left its buffer
    if (s->used[slot]) MZ_CK(cudaStreamWaitEvent(c->stream, s->done[slot], 0));
    double* b = s->buf[slot];
    MZ_CK(cudaMemcpyAsync(b, p->np, m * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    MZ_CK(cudaMemcpyAsync(b + m, p->n, m * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    MZ_CK(cudaMemcpyAsync(b + 2 * m, p->v, 3 * m * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    MZ_CK(cudaMemcpyAsync(b + 5 * m, p->T, m * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    MZ_CK(cudaEventRecord(s->ready[slot], c->stream));
    MZ_CK(cudaStreamWaitEvent(s->side, s->ready[slot], 0));
    MZ_CK(cudaMemcpyAsync(dst, b, s->doubles * sizeof(double), cudaMemcpyDeviceToHost, s->side));
    MZ_CK(cudaEventRecord(s->done[slot], s->side));
    s->used[slot] = true;
    API_CATCH(p ? p->dom->ctx : nullptr)
}

int mz_props_snapshot_wait(mz_props* p, int32_t slot)
{
    API_TRY
    MZ_REQUIRE(p && (slot == 0 || slot == 1), "mz_props_snapshot_wait: bad argument");
    PropsSnapshot* s = static_cast<PropsSnapshot*>(p->snapshot);
    if (!s || !s->used[slot]) return MZ_OK;
    MZ_CK(cudaSetDevice(p->dom->ctx->device));
    MZ_CK(cudaEventSynchronize(s->done[slot]));
    API_CATCH(p ? p->dom->ctx : nullptr)
}

int mz_host_alloc(mz_ctx* c, size_t bytes, void** out)
{
    API_TRY
    MZ_REQUIRE(c && out && bytes > 0, "mz_host_alloc: bad argument");
    MZ_CK(cudaSetDevice(c->device));
    *out = nullptr;
    MZ_CK(cudaMallocHost(out, bytes));
    API_CATCH(c)
}

int mz_host_free(void* ptr)
{
    if (ptr) cudaFreeHost(ptr);
    return MZ_OK;
}

}  // extern "C"
