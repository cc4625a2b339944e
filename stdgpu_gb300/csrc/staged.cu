// Table calls on HOST buffers: the inputs stream in through a ring of device staging buffers while
// the kernels of earlier chunks run, and the outputs stream back the same way.
//
// The reference's bulk calls take device iterators only (src/stdgpu/impl/unordered_base_detail.cuh:
// 996-1066), so a caller holding its keys in host memory copies them in first, runs the call, and
// copies the results out: three serial phases.  Here a call is cut into chunks; chunk c is copied
// host->device on the stager's upload stream into buffer c mod B, the table kernel for chunk c runs on
// the caller's stream once that copy is done, and its results go device->host on the download stream
// while chunk c+1 is processed.  Buffer reuse is ordered by events (a buffer is refilled only after its
// previous chunk's kernel and download finished), so at most B chunks are in flight.
//
// Ordering seen by the caller: every copy of a call starts after the work already queued on the
// caller's stream (unless the caller declared its inputs ready, sg_stager_set_inputs_ready: then the
// uploads start at once and only the kernels keep stream order), and the caller's stream waits for the
// call's last download, so a call behaves like one stream-ordered operation.  The host buffers must stay valid until then; with pinned memory
// (cudaHostAlloc / cudaHostRegister) the copies are asynchronous, with pageable memory they still work
// but do not overlap the kernels.
#include <cuda_runtime.h>

#include <cstdint>
#include <new>

#include "sg_internal.cuh"
#include "stdgpu_gb300.h"

namespace
{

constexpr int kMaxBuffers = 8;
constexpr int64_t kAlign = 256;

int64_t
round_up(int64_t x)
{
    return (x + kAlign - 1) / kAlign * kAlign;
}

} // namespace

struct sg_stager
{
    int64_t chunk = 0;
    int32_t n_buffers = 0;
    int32_t next = 0;
    int device = 0;
    char* mem = nullptr;          // n_buffers x per-buffer bytes
    int64_t buffer_bytes = 0;
    int64_t off_in1 = 0;          // offsets inside one buffer: in0 (16 B / element), in1 (8 B), out0 (8 B), out1 (1 B)
    int64_t off_out0 = 0;
    int64_t off_out1 = 0;
    cudaStream_t up = nullptr;
    cudaStream_t down = nullptr;
    cudaEvent_t start = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t ready[kMaxBuffers] = {};
    cudaEvent_t used[kMaxBuffers] = {};
    cudaEvent_t freed[kMaxBuffers] = {};
    bool inputs_ready = false; // uploads need not wait for the caller's earlier work
};

namespace
{

struct host_in
{
    const void* ptr;
    int32_t bytes; // per element
};

struct host_out
{
    void* ptr;
    int32_t bytes;
};

// Element sizes of a table's kind: value_type, key, mapped.
sg_status
kind_sizes(const sg_unordered* t, int32_t* value_bytes, int32_t* key_bytes, int32_t* mapped_bytes)
{
    sg_unordered_view v{};
    const sg_status st = sg_unordered_view_of(t, &v);
    if (st != SG_OK)
    {
        return st;
    }
    switch (v.kind)
    {
        case SG_SET_U32: *value_bytes = 4; *key_bytes = 4; *mapped_bytes = 0; break;
        case SG_SET_U64: *value_bytes = 8; *key_bytes = 8; *mapped_bytes = 0; break;
        case SG_MAP_U64_U32: *value_bytes = 16; *key_bytes = 8; *mapped_bytes = 4; break;
        case SG_MAP_U64_U64: *value_bytes = 16; *key_bytes = 8; *mapped_bytes = 8; break;
        case SG_MAP_U32_U32: *value_bytes = 8; *key_bytes = 4; *mapped_bytes = 4; break;
        case SG_MAP_U32_U64: *value_bytes = 16; *key_bytes = 4; *mapped_bytes = 8; break;
        default: return SG_ERR_BAD_ARG;
    }
    return SG_OK;
}

// Runs `launch(in0, in1, out0, out1, m, stream)` over chunks of n elements; null host pointers stay null.
template <typename Launch>
sg_status
staged(sg_stager* sg, cudaStream_t s, int64_t n, host_in in0, host_in in1, host_out out0, host_out out1,
       Launch launch)
{
    int dev = -1;
    SG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev != sg->device)
    {
        return SG_ERR_BAD_ARG;
    }
    const bool any_out = out0.ptr != nullptr || out1.ptr != nullptr;
    if (!sg->inputs_ready)
    {
        SG_CUDA_TRY(cudaEventRecord(sg->start, s));
        SG_CUDA_TRY(cudaStreamWaitEvent(sg->up, sg->start, 0));
    }
    for (int64_t off = 0; off < n; off += sg->chunk)
    {
        const int64_t m = n - off < sg->chunk ? n - off : sg->chunk;
        const int b = sg->next;
        sg->next = (b + 1) % sg->n_buffers;
        char* base = sg->mem + static_cast<int64_t>(b) * sg->buffer_bytes;
        void* d_in0 = in0.ptr != nullptr ? base : nullptr;
        void* d_in1 = in1.ptr != nullptr ? base + sg->off_in1 : nullptr;
        void* d_out0 = out0.ptr != nullptr ? base + sg->off_out0 : nullptr;
        uint8_t* d_out1 = out1.ptr != nullptr ? reinterpret_cast<uint8_t*>(base + sg->off_out1) : nullptr;

        SG_CUDA_TRY(cudaStreamWaitEvent(sg->up, sg->freed[b], 0));
        if (d_in0 != nullptr)
        {
            SG_CUDA_TRY(cudaMemcpyAsync(d_in0, static_cast<const char*>(in0.ptr) + off * in0.bytes, m * in0.bytes,
                                        cudaMemcpyHostToDevice, sg->up));
        }
        if (d_in1 != nullptr)
        {
            SG_CUDA_TRY(cudaMemcpyAsync(d_in1, static_cast<const char*>(in1.ptr) + off * in1.bytes, m * in1.bytes,
                                        cudaMemcpyHostToDevice, sg->up));
        }
        SG_CUDA_TRY(cudaEventRecord(sg->ready[b], sg->up));
        SG_CUDA_TRY(cudaStreamWaitEvent(s, sg->ready[b], 0));
        const sg_status st = launch(d_in0, d_in1, d_out0, d_out1, m, s);
        if (st != SG_OK)
        {
            return st;
        }
        if (any_out)
        {
            SG_CUDA_TRY(cudaEventRecord(sg->used[b], s));
            SG_CUDA_TRY(cudaStreamWaitEvent(sg->down, sg->used[b], 0));
            if (d_out0 != nullptr)
            {
                SG_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(out0.ptr) + off * out0.bytes, d_out0, m * out0.bytes,
                                            cudaMemcpyDeviceToHost, sg->down));
            }
            if (d_out1 != nullptr)
            {
                SG_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(out1.ptr) + off * out1.bytes, d_out1, m * out1.bytes,
                                            cudaMemcpyDeviceToHost, sg->down));
            }
            SG_CUDA_TRY(cudaEventRecord(sg->freed[b], sg->down));
        }
        else
        {
            SG_CUDA_TRY(cudaEventRecord(sg->freed[b], s));
        }
    }
    if (any_out)
    {
        SG_CUDA_TRY(cudaEventRecord(sg->done, sg->down));
        SG_CUDA_TRY(cudaStreamWaitEvent(s, sg->done, 0));
    }
    return SG_OK;
}

} // namespace

extern "C" {

sg_status
sg_stager_create(int64_t chunk_elems, int32_t n_buffers, sg_stager** out)
{
    if (out == nullptr || chunk_elems <= 0 || chunk_elems > (int64_t{ 1 } << 30) || n_buffers < 2 ||
        n_buffers > kMaxBuffers)
    {
        return SG_ERR_BAD_ARG;
    }
    *out = nullptr;
    auto* sg = new (std::nothrow) sg_stager{};
    if (sg == nullptr)
    {
        return SG_ERR_OOM;
    }
    sg->chunk = chunk_elems;
    sg->n_buffers = n_buffers;
    sg->off_in1 = round_up(chunk_elems * 16);
    sg->off_out0 = sg->off_in1 + round_up(chunk_elems * 8);
    sg->off_out1 = sg->off_out0 + round_up(chunk_elems * 8);
    sg->buffer_bytes = sg->off_out1 + round_up(chunk_elems);
    cudaError_t e = cudaGetDevice(&sg->device);
    if (e == cudaSuccess)
    {
        e = sg::detail::dev_malloc(reinterpret_cast<void**>(&sg->mem), static_cast<size_t>(sg->buffer_bytes) * n_buffers);
    }
    if (e == cudaSuccess)
    {
        e = cudaStreamCreateWithFlags(&sg->up, cudaStreamNonBlocking);
    }
    if (e == cudaSuccess)
    {
        e = cudaStreamCreateWithFlags(&sg->down, cudaStreamNonBlocking);
    }
    if (e == cudaSuccess)
    {
        e = cudaEventCreateWithFlags(&sg->start, cudaEventDisableTiming);
    }
    if (e == cudaSuccess)
    {
        e = cudaEventCreateWithFlags(&sg->done, cudaEventDisableTiming);
    }
    for (int b = 0; b < n_buffers && e == cudaSuccess; ++b)
    {
        e = cudaEventCreateWithFlags(&sg->ready[b], cudaEventDisableTiming);
        if (e == cudaSuccess)
        {
            e = cudaEventCreateWithFlags(&sg->used[b], cudaEventDisableTiming);
        }
        if (e == cudaSuccess)
        {
            e = cudaEventCreateWithFlags(&sg->freed[b], cudaEventDisableTiming);
        }
    }
    if (e != cudaSuccess)
    {
        sg_stager_destroy(sg);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA;
    }
    *out = sg;
    return SG_OK;
}

sg_status
sg_stager_destroy(sg_stager* sg)
{
    if (sg == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    if (sg->up != nullptr)
    {
        cudaStreamSynchronize(sg->up);
    }
    if (sg->down != nullptr)
    {
        cudaStreamSynchronize(sg->down);
    }
    for (int b = 0; b < kMaxBuffers; ++b)
    {
        // a buffer's last kernel may still run on a caller's stream
        if (sg->freed[b] != nullptr)
        {
            cudaEventSynchronize(sg->freed[b]);
        }
    }
    for (int b = 0; b < kMaxBuffers; ++b)
    {
        if (sg->ready[b] != nullptr)
        {
            cudaEventDestroy(sg->ready[b]);
        }
        if (sg->used[b] != nullptr)
        {
            cudaEventDestroy(sg->used[b]);
        }
        if (sg->freed[b] != nullptr)
        {
            cudaEventDestroy(sg->freed[b]);
        }
    }
    if (sg->start != nullptr)
    {
        cudaEventDestroy(sg->start);
    }
    if (sg->done != nullptr)
    {
        cudaEventDestroy(sg->done);
    }
    if (sg->up != nullptr)
    {
        cudaStreamDestroy(sg->up);
    }
    if (sg->down != nullptr)
    {
        cudaStreamDestroy(sg->down);
    }
    sg::detail::dev_free(sg->mem);
    delete sg;
    return SG_OK;
}

sg_status
sg_stager_set_inputs_ready(sg_stager* sg, int32_t inputs_ready)
{
    if (sg == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    sg->inputs_ready = inputs_ready != 0;
    return SG_OK;
}

sg_status
sg_unordered_insert_host(sg_unordered* t, sg_stager* sg, const void* values, int64_t n, uint8_t* out_inserted,
                         void* stream)
{
    int32_t vb = 0, kb = 0, mb = 0;
    if (t == nullptr || sg == nullptr || n < 0 || (n > 0 && values == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    const sg_status ks = kind_sizes(t, &vb, &kb, &mb);
    if (ks != SG_OK)
    {
        return ks;
    }
    return staged(sg, sg::detail::as_stream(stream), n, { values, vb }, { nullptr, 0 }, { nullptr, 0 },
                  { out_inserted, 1 },
                  [t](void* in0, void*, void*, uint8_t* out1, int64_t m, cudaStream_t s)
                  { return sg_unordered_insert(t, in0, m, out1, s); });
}

sg_status
sg_unordered_insert_kv_host(sg_unordered* t, sg_stager* sg, const void* keys, const void* mapped, int64_t n,
                            uint8_t* out_inserted, void* stream)
{
    int32_t vb = 0, kb = 0, mb = 0;
    if (t == nullptr || sg == nullptr || n < 0 || (n > 0 && keys == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    const sg_status ks = kind_sizes(t, &vb, &kb, &mb);
    if (ks != SG_OK)
    {
        return ks;
    }
    const void* m_in = mb > 0 ? mapped : nullptr;
    return staged(sg, sg::detail::as_stream(stream), n, { keys, kb }, { m_in, mb }, { nullptr, 0 },
                  { out_inserted, 1 },
                  [t](void* in0, void* in1, void*, uint8_t* out1, int64_t m, cudaStream_t s)
                  { return sg_unordered_insert_kv(t, in0, in1, m, out1, s); });
}

sg_status
sg_unordered_erase_host(sg_unordered* t, sg_stager* sg, const void* keys, int64_t n, uint8_t* out_erased,
                        void* stream)
{
    int32_t vb = 0, kb = 0, mb = 0;
    if (t == nullptr || sg == nullptr || n < 0 || (n > 0 && keys == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    const sg_status ks = kind_sizes(t, &vb, &kb, &mb);
    if (ks != SG_OK)
    {
        return ks;
    }
    return staged(sg, sg::detail::as_stream(stream), n, { keys, kb }, { nullptr, 0 }, { nullptr, 0 },
                  { out_erased, 1 },
                  [t](void* in0, void*, void*, uint8_t* out1, int64_t m, cudaStream_t s)
                  { return sg_unordered_erase(t, in0, m, out1, s); });
}

sg_status
sg_unordered_find_host(sg_unordered* t, sg_stager* sg, const void* keys, int64_t n, void* out_mapped,
                       uint8_t* out_found, void* stream)
{
    int32_t vb = 0, kb = 0, mb = 0;
    if (t == nullptr || sg == nullptr || n < 0 || (n > 0 && keys == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    const sg_status ks = kind_sizes(t, &vb, &kb, &mb);
    if (ks != SG_OK)
    {
        return ks;
    }
    void* mo = mb > 0 ? out_mapped : nullptr;
    return staged(sg, sg::detail::as_stream(stream), n, { keys, kb }, { nullptr, 0 }, { mo, mb }, { out_found, 1 },
                  [t, mb](void* in0, void*, void* out0, uint8_t* out1, int64_t m, cudaStream_t s)
                  {
                      // the staging buffer holds an earlier chunk's values: absent keys read back as 0
                      if (out0 != nullptr)
                      {
                          SG_CUDA_TRY(cudaMemsetAsync(out0, 0, static_cast<size_t>(m) * mb, s));
                      }
                      return sg_unordered_find(t, in0, m, out0, out1, s);
                  });
}

sg_status
sg_unordered_contains_host(sg_unordered* t, sg_stager* sg, const void* keys, int64_t n, uint8_t* out_flags,
                           void* stream)
{
    int32_t vb = 0, kb = 0, mb = 0;
    if (t == nullptr || sg == nullptr || n < 0 || (n > 0 && keys == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    const sg_status ks = kind_sizes(t, &vb, &kb, &mb);
    if (ks != SG_OK)
    {
        return ks;
    }
    return staged(sg, sg::detail::as_stream(stream), n, { keys, kb }, { nullptr, 0 }, { nullptr, 0 },
                  { out_flags, 1 },
                  [t](void* in0, void*, void*, uint8_t* out1, int64_t m, cudaStream_t s)
                  { return sg_unordered_contains(t, in0, m, out1, s); });
}

} // extern "C"
