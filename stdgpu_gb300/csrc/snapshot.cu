// Table snapshots (save / load) and rehash into a new capacity.  The reference has neither: its capacity
// is fixed at creation (src/stdgpu/unordered_map.cuh:61) and it has no on-disk form; a served or
// checkpointed table needs both.
//
// Snapshot file: a 128-byte header (magic, format version, kind, custom-hash flag, the creation capacity
// and the geometry it implies, the byte counts that follow), then the device header of the table, then the
// raw slot image -- every 128-byte probe group plus the out-of-band tail group.  Loading recreates the
// table from the capacity, checks that the geometry matches, and copies the image back, so the restored
// table is bit for bit the saved one (erased slots included), whatever the keys' hash function.  A table
// with the reference's excess-list accounting on (format version 2) also stores its two bit arrays after the
// image; a version-1 file loads with the accounting off.
// Copies go through one pinned staging buffer in 64 MB pieces.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>

#include "sg_internal.cuh"
#include "stdgpu_gb300.h"
#include "stdgpu_gb300/detail/layout.cuh"

namespace
{

constexpr char kMagic[8] = { 'S', 'G', 'G', 'B', '3', '0', '0', 'T' };
constexpr uint32_t kVersion = 2;
constexpr size_t kPiece = size_t{ 64 } << 20;

struct file_header
{
    char magic[8];
    uint32_t version;
    int32_t kind;
    uint32_t custom_hash;
    uint32_t slot_bytes;
    int64_t capacity;
    int64_t bucket_count;
    int64_t max_size;
    int64_t num_groups;
    int64_t header_bytes; // device table header
    int64_t image_bytes;  // probe groups + tail group
    int64_t bucket_heads_bytes; // excess-list accounting (version 2): 0 when off
    int64_t slot_heads_bytes;
    uint8_t reserved[128 - 8 - 16 - 8 * 8];
};
static_assert(sizeof(file_header) == 128, "128-byte file header");

struct pinned
{
    void* p = nullptr;
    pinned() { cudaMallocHost(&p, kPiece); }
    ~pinned()
    {
        if (p != nullptr)
        {
            cudaFreeHost(p);
        }
    }
};

sg_status
device_to_file(const void* src, int64_t bytes, std::FILE* f, cudaStream_t s, pinned& buf)
{
    const char* d = static_cast<const char*>(src);
    for (int64_t off = 0; off < bytes; off += static_cast<int64_t>(kPiece))
    {
        const size_t m = static_cast<size_t>(bytes - off < static_cast<int64_t>(kPiece) ? bytes - off : kPiece);
        SG_CUDA_TRY(cudaMemcpyAsync(buf.p, d + off, m, cudaMemcpyDeviceToHost, s));
        SG_CUDA_TRY(cudaStreamSynchronize(s));
        if (std::fwrite(buf.p, 1, m, f) != m)
        {
            return SG_ERR_BAD_ARG;
        }
    }
    return SG_OK;
}

sg_status
file_to_device(void* dst, int64_t bytes, std::FILE* f, cudaStream_t s, pinned& buf)
{
    char* d = static_cast<char*>(dst);
    for (int64_t off = 0; off < bytes; off += static_cast<int64_t>(kPiece))
    {
        const size_t m = static_cast<size_t>(bytes - off < static_cast<int64_t>(kPiece) ? bytes - off : kPiece);
        if (std::fread(buf.p, 1, m, f) != m)
        {
            return SG_ERR_BAD_ARG;
        }
        SG_CUDA_TRY(cudaMemcpyAsync(d + off, buf.p, m, cudaMemcpyHostToDevice, s));
        SG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SG_OK;
}

struct file_closer
{
    std::FILE* f;
    ~file_closer()
    {
        if (f != nullptr)
        {
            std::fclose(f);
        }
    }
};

} // namespace

extern "C" {

sg_status
sg_unordered_save(sg_unordered* t, const char* path, void* stream)
{
    if (t == nullptr || path == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    sg_unordered_view v{};
    sg_geometry g{};
    sg_status st = sg_unordered_view_of(t, &v);
    if (st == SG_OK)
    {
        st = sg_unordered_geometry(t, &g);
    }
    int32_t custom = 0;
    if (st == SG_OK)
    {
        st = sg_unordered_is_hashed(t, &custom);
    }
    if (st != SG_OK)
    {
        return st;
    }
    file_header h{};
    std::memcpy(h.magic, kMagic, sizeof(kMagic));
    h.version = kVersion;
    h.kind = v.kind;
    h.custom_hash = static_cast<uint32_t>(custom);
    h.slot_bytes = static_cast<uint32_t>(g.slot_bytes);
    h.capacity = g.capacity;
    h.bucket_count = g.bucket_count;
    h.max_size = g.max_size;
    h.num_groups = g.num_groups;
    h.header_bytes = static_cast<int64_t>(sizeof(sg::detail::table_header));
    h.image_bytes = (g.num_groups + 1) * sg::detail::kGroupBytes;
    if (v.bucket_heads != nullptr)
    {
        h.bucket_heads_bytes = (v.bucket_count + 31) / 32 * 4;
        h.slot_heads_bytes = (v.num_groups * g.slots_per_group + 2 + 31) / 32 * 4;
    }
    file_closer fc{ std::fopen(path, "wb") };
    if (fc.f == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    if (std::fwrite(&h, sizeof(h), 1, fc.f) != 1)
    {
        return SG_ERR_BAD_ARG;
    }
    pinned buf;
    if (buf.p == nullptr)
    {
        return SG_ERR_OOM;
    }
    cudaStream_t s = sg::detail::as_stream(stream);
    st = device_to_file(v.header, h.header_bytes, fc.f, s, buf);
    if (st != SG_OK)
    {
        return st;
    }
    st = device_to_file(v.slots, h.image_bytes, fc.f, s, buf);
    if (st == SG_OK && v.bucket_heads != nullptr)
    {
        st = device_to_file(v.bucket_heads, h.bucket_heads_bytes, fc.f, s, buf);
        if (st == SG_OK)
        {
            st = device_to_file(v.slot_heads, h.slot_heads_bytes, fc.f, s, buf);
        }
    }
    return st;
}

sg_status
sg_unordered_load(const char* path, void* stream, sg_unordered** out)
{
    if (path == nullptr || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    *out = nullptr;
    file_closer fc{ std::fopen(path, "rb") };
    if (fc.f == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    file_header h{};
    if (std::fread(&h, sizeof(h), 1, fc.f) != 1 || std::memcmp(h.magic, kMagic, sizeof(kMagic)) != 0 ||
        h.version < 1 || h.version > kVersion)
    {
        return SG_ERR_BAD_ARG;
    }
    if (h.version == 1)
    {
        h.bucket_heads_bytes = 0;
        h.slot_heads_bytes = 0;
    }
    // the file must describe exactly the table that createDeviceObject(capacity) builds
    sg_geometry g{};
    if (sg_unordered_geometry_for(h.kind, h.capacity, &g) != SG_OK || g.bucket_count != h.bucket_count ||
        g.max_size != h.max_size || g.num_groups != h.num_groups || g.slot_bytes != static_cast<int32_t>(h.slot_bytes) ||
        h.header_bytes != static_cast<int64_t>(sizeof(sg::detail::table_header)) ||
        h.image_bytes != (g.num_groups + 1) * sg::detail::kGroupBytes || h.custom_hash > 1)
    {
        return SG_ERR_BAD_ARG;
    }
    const bool accounting = h.bucket_heads_bytes != 0;
    if (accounting && (h.bucket_heads_bytes != (g.bucket_count + 31) / 32 * 4 ||
                       h.slot_heads_bytes != (g.num_groups * g.slots_per_group + 2 + 31) / 32 * 4))
    {
        return SG_ERR_BAD_ARG;
    }
    sg_unordered* t = nullptr;
    sg_status st = h.custom_hash != 0 ? sg_unordered_create_hashed(h.kind, h.capacity, stream, &t)
                                      : sg_unordered_create(h.kind, h.capacity, stream, &t);
    if (st != SG_OK)
    {
        return st;
    }
    st = sg_unordered_set_excess_accounting(t, accounting ? 1 : 0, stream);
    if (st != SG_OK)
    {
        sg_unordered_destroy(t);
        return st;
    }
    sg_unordered_view v{};
    sg_unordered_view_of(t, &v);
    pinned buf;
    if (buf.p == nullptr)
    {
        sg_unordered_destroy(t);
        return SG_ERR_OOM;
    }
    cudaStream_t s = sg::detail::as_stream(stream);
    st = file_to_device(v.header, h.header_bytes, fc.f, s, buf);
    if (st == SG_OK)
    {
        st = file_to_device(v.slots, h.image_bytes, fc.f, s, buf);
    }
    if (st == SG_OK && accounting)
    {
        st = file_to_device(v.bucket_heads, h.bucket_heads_bytes, fc.f, s, buf);
        if (st == SG_OK)
        {
            st = file_to_device(v.slot_heads, h.slot_heads_bytes, fc.f, s, buf);
        }
    }
    if (st != SG_OK)
    {
        sg_unordered_destroy(t);
        return st;
    }
    *out = t;
    return SG_OK;
}

} // extern "C"
