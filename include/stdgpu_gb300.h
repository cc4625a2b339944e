/*
 * stdgpu_gb300 -- C ABI of the GB300 (sm_103a) hashed-container path.
 *
 * Plain C: opaque handles, plain pointers and sizes, `void*` for a CUDA stream
 * (a cudaStream_t; NULL = the legacy default stream).  Every data pointer is a
 * DEVICE pointer owned by the caller.  Calls are stream-ordered and
 * asynchronous unless they return a host value through an out-parameter (those
 * synchronise the given stream).  Distinct handles may be used concurrently on
 * distinct streams; one handle must not be used from two host threads at once.
 *
 * Errors are returned as sg_status codes; no entry point aborts the process
 * (the reference calls std::terminate on CUDA errors,
 * src/stdgpu/cuda/impl/error.h:41-56).  Device-side conditions that the
 * reference only printf()s (a refused insert into a full table, a bounded wait
 * that ran out) are counted on the device and reported by the next call that
 * synchronises (sg_unordered_size, sg_unordered_valid, ...).
 *
 * Each entry point cites the reference interface it replaces (paths relative
 * to the stdgpu 1.3.0 source tree).
 */
#ifndef STDGPU_GB300_H
#define STDGPU_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SG_API __attribute__((visibility("default")))
#else
#define SG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sg_status
{
    SG_OK = 0,
    SG_ERR_FULL = 1,             /* inserts were refused because the table / container was full */
    SG_ERR_BAD_ARG = 2,          /* null handle, negative size, unknown kind, size above a limit */
    SG_ERR_OOM = 3,              /* device allocation failed */
    SG_ERR_BUDGET = 4,           /* refused by an HBM budget (serving / batched entry points) */
    SG_ERR_RETRY_EXHAUSTED = 5,  /* a bounded device wait or retry loop gave up */
    SG_ERR_CUDA = 6,             /* a CUDA runtime call failed */
    SG_ERR_NO_DEVICE = 7         /* no usable sm_103 device */
} sg_status;

/* Container kinds: key type and mapped type of unordered_set<Key> / unordered_map<Key,T>.
 * The element layout in device memory is that of the reference's value_type:
 * Key for sets, stdgpu::pair<const Key, T> for maps (src/stdgpu/unordered_map.cuh:80,
 * src/stdgpu/unordered_set.cuh:69), i.e. key at offset 0 and T at its natural alignment. */
typedef enum sg_kind
{
    SG_SET_U32 = 0,     /* unordered_set<uint32_t>            element  4 B */
    SG_SET_U64 = 1,     /* unordered_set<uint64_t>            element  8 B */
    SG_MAP_U64_U32 = 2, /* unordered_map<uint64_t, uint32_t>  element 16 B */
    SG_MAP_U64_U64 = 3, /* unordered_map<uint64_t, uint64_t>  element 16 B */
    SG_MAP_U32_U32 = 4, /* unordered_map<uint32_t, uint32_t>  element  8 B */
    SG_MAP_U32_U64 = 5  /* unordered_map<uint32_t, uint64_t>  element 16 B */
} sg_kind;

typedef struct sg_unordered sg_unordered;

/* Geometry of a table.  bucket_count / excess_count / max_size follow the reference's
 * createDeviceObject (src/stdgpu/impl/unordered_base_detail.cuh:1264-1273); the rest
 * describes this implementation's storage. */
typedef struct sg_geometry
{
    int64_t capacity;        /* as passed to create */
    int64_t bucket_count;    /* bucket_count()   unordered_base_detail.cuh:1141-1146 */
    int64_t excess_count;    /* expected_collisions(bucket_count, capacity) + 1 */
    int64_t max_size;        /* max_size() = total_count = bucket_count + excess_count */
    int64_t num_groups;      /* 128-byte probe groups */
    int32_t slot_bytes;      /* sizeof(value_type) */
    int32_t slots_per_group; /* 128 / slot_bytes */
    int64_t storage_bytes;   /* device bytes held by the table */
} sg_geometry;

/* Device view of a table for native device calls (include/stdgpu_gb300/device.cuh).
 * Plain data; copy it by value into kernels. */
typedef struct sg_unordered_view
{
    void* slots;             /* (num_groups + 1) * 128 bytes; the last group holds the two out-of-band keys */
    void* header;            /* device counters */
    int64_t num_groups;
    int64_t total_count;     /* max_size(); slots at or above this index are never used */
    int64_t bucket_count;
    int32_t bucket_bits;     /* log2(bucket_count) */
    int32_t kind;
    uint32_t* insert_locks;  /* device stripe locks of the native device inserts, lock_mask + 1 of them (a power
                                of two); nullable: device inserts then claim never-used slots only */
    int64_t lock_mask;
    /* The reference's excess-list accounting (NULL: off).  The reference stores a new key in its bucket's own
     * slot when that slot is free, else in a slot taken from its excess list, and refuses every insert once
     * that list is empty (unordered_base_detail.cuh:708-809, 958-994); these fields track the same state. */
    uint32_t* bucket_heads;  /* one bit per bucket: set while a key holds the bucket's own slot */
    uint32_t* slot_heads;    /* one bit per slot (num_groups x slots per group, then the 2 out-of-band slots):
                                set where the key holding its bucket's own slot is stored */
    int64_t excess_count;    /* the excess list's length */
} sg_unordered_view;

/* ---------------- device memory ---------------- */

/* The allocator of every container's device storage (the reference's Allocator template parameter,
 * src/stdgpu/memory.h; safe_device_allocator by default).  alloc returns device memory of at least `bytes`
 * (NULL when it cannot), release gives it back; both get ctx.  Passing NULL for both restores
 * cudaMalloc / cudaFree.  SG_ERR_BAD_ARG (nothing changed) while storage made through the current pair is
 * still allocated, or when only one of the two functions is given.  Pinned host buffers are not
 * affected. */
typedef void* (*sg_device_alloc_fn)(size_t bytes, void* ctx);
typedef void (*sg_device_free_fn)(void* ptr, void* ctx);
SG_API sg_status sg_set_device_allocator(sg_device_alloc_fn alloc, sg_device_free_fn release, void* ctx);
/* Number of device allocations the library holds (all containers, staging and scratch buffers). */
SG_API int64_t sg_live_device_allocations(void);

/* An allocator of one table's device storage: the reference's Allocator argument of
 * createDeviceObject(capacity, allocator) (src/stdgpu/impl/unordered_base_detail.cuh:1254-1308 allocates
 * the table's arrays through it with allocator_traits).  Every device allocation the table makes in its
 * life -- slots, header, counters, bulk-call scratch, the storage a rehash rebuilds -- goes through
 * alloc / release with ctx (a release is preceded by a device synchronisation, as cudaFree is), and
 * release_ctx (nullable) is called with ctx once the table is destroyed.  The memory must be device memory
 * of the current device.  These allocations are not counted by sg_live_device_allocations. */
typedef struct sg_allocator
{
    sg_device_alloc_fn alloc;
    sg_device_free_fn release;
    void* ctx;
    void (*release_ctx)(void* ctx);
} sg_allocator;

/* ---------------- unordered_set / unordered_map ---------------- */

/* createDeviceObject(capacity): src/stdgpu/impl/unordered_base_detail.cuh:1254-1308,
 * src/stdgpu/impl/unordered_map_detail.cuh:397-419.  capacity > 0 and max_size() < 2^31
 * (the reference's 32-bit index_t, src/stdgpu/cstddef.h:42-59). */
SG_API sg_status sg_unordered_create(int32_t kind, int64_t capacity, void* stream, sg_unordered** out);

/* destroyDeviceObject: src/stdgpu/impl/unordered_base_detail.cuh:1310-1348 */
SG_API sg_status sg_unordered_destroy(sg_unordered* table);
/* createDeviceObject(capacity, allocator): sg_unordered_create (custom_hash = 0) or sg_unordered_create_hashed
 * (custom_hash = 1) with the table's storage taken from `allocator` (copied; alloc and release non-null). */
SG_API sg_status sg_unordered_create_with_allocator(int32_t kind, int64_t capacity, int32_t custom_hash,
                                                    const sg_allocator* allocator, void* stream, sg_unordered** out);

/* insert(begin, end) with begin pointing at value_type elements:
 * src/stdgpu/impl/unordered_base_detail.cuh:996-1017 (per element :967-994).
 * out_inserted (nullable): per element 1 if this element was inserted, else 0. */
SG_API sg_status sg_unordered_insert(sg_unordered* table, const void* values, int64_t n, uint8_t* out_inserted,
                              void* stream);

/* Same as sg_unordered_insert with keys and mapped values in two arrays (mapped ignored for sets). */
SG_API sg_status sg_unordered_insert_kv(sg_unordered* table, const void* keys, const void* mapped, int64_t n,
                                 uint8_t* out_inserted, void* stream);

/* ---- Custom key types and hash functions: unordered_set<Key, Hash> / unordered_map<Key, T, Hash>
 * (src/stdgpu/unordered_map.cuh:70-80, unordered_set.cuh:61-69 with a user Hash; the reference's own tests use
 * vec3int16 keys with vec_hash, tests/stdgpu/unordered_map.inc:178-206).  A key of at most 8 bytes whose
 * equality is equality of its bytes (short3, vec3int16, packed coordinates) is stored as a zero-padded
 * 4- or 8-byte key word, so the table is one of the six kinds; the bucket of a key is the fibonacci hashing
 * of Hash(key) (unordered_base_detail.cuh:56-85), which the caller computes (the C++ API in
 * stdgpu_gb300/stdgpu.cuh does it with the user's functor) and passes per key as a 64-bit hash.  A table
 * created this way takes only the *_hashed bulk calls (the identity-hash calls return SG_ERR_BAD_ARG), and
 * sg_unordered_valid checks it without re-deriving buckets (reachability needs the hash). */
SG_API sg_status sg_unordered_create_hashed(int32_t kind, int64_t capacity, void* stream, sg_unordered** out);
SG_API sg_status sg_unordered_insert_hashed(sg_unordered* table, const void* keys, const void* mapped,
                                            const uint64_t* hashes, int64_t n, uint8_t* out_inserted, void* stream);
SG_API sg_status sg_unordered_erase_hashed(sg_unordered* table, const void* keys, const uint64_t* hashes, int64_t n,
                                           uint8_t* out_erased, void* stream);
SG_API sg_status sg_unordered_find_hashed(sg_unordered* table, const void* keys, const uint64_t* hashes, int64_t n,
                                          void* out_mapped, uint8_t* out_found, void* stream);
SG_API sg_status sg_unordered_contains_hashed(sg_unordered* table, const void* keys, const uint64_t* hashes,
                                              int64_t n, uint8_t* out_flags, void* stream);
/* bucket() of a key whose hash is `hash`: fibonacci hashing onto bucket_count (unordered_base_detail.cuh:547-564). */
SG_API sg_status sg_unordered_bucket_of_hash(const sg_unordered* table, uint64_t hash, int64_t* out_bucket);

/* 1 when the table was created by sg_unordered_create_hashed. */
SG_API sg_status sg_unordered_is_hashed(const sg_unordered* table, int32_t* out);

/* ---- Rehash and snapshots (no counterpart in the reference: its capacity is fixed at creation,
 * src/stdgpu/unordered_map.cuh:61, and it has no on-disk form).
 * rehash: moves every element into storage built for new_capacity (the geometry of
 * createDeviceObject(new_capacity)); the handle stays valid, views taken before it do not.  Synchronises.
 * SG_ERR_FULL (table unchanged) when the elements do not fit; SG_ERR_BAD_ARG on a custom-hash table.
 * save / load: a binary file holding the creation capacity, the geometry and the raw image of the table
 * (device header, every probe group), so a loaded table is bit for bit the saved one; load checks the
 * header and the geometry before it allocates anything.  Both synchronise. */
SG_API sg_status sg_unordered_rehash(sg_unordered* table, int64_t new_capacity, void* stream);
SG_API sg_status sg_unordered_save(sg_unordered* table, const char* path, void* stream);
SG_API sg_status sg_unordered_load(const char* path, void* stream, sg_unordered** out);

/* Bulk-insert strategy (no counterpart in the reference).  SG_INSERT_AUTO: when a call without per-element
 * flags brings at least 2^22 keys and one key per two probe groups of a table of 256 MB or more, the keys
 * are first partitioned by home-group range, in one pass, into a scratch array (about 1.13 x n x
 * sizeof(value_type): each range's share plus slack and an overflow region; kept by the table until
 * destroy) so that each group line is read from DRAM about once; elements that find no room there (keys
 * crowded into few ranges) are inserted by a direct pass over the whole input.  Bulk erase partitions its
 * keys the same way from 2^22 keys on.  SG_INSERT_DIRECT never partitions; SG_INSERT_PARTITIONED
 * partitions every call without flags.  Results are the same. */
typedef enum sg_insert_mode
{
    SG_INSERT_AUTO = 0,
    SG_INSERT_DIRECT = 1,
    SG_INSERT_PARTITIONED = 2
} sg_insert_mode;
SG_API sg_status sg_unordered_set_insert_mode(sg_unordered* table, int32_t mode);

/* The reference's excess-list refusal.  The reference keeps a new key in its bucket's own slot when that is
 * free, else in a slot of its excess list (excess_count slots), and its insert loop refuses every insert
 * once that list is empty or the table is full (src/stdgpu/impl/unordered_base_detail.cuh:708-809, 958-994),
 * which can happen below max_size().  With the accounting on (on = 1), a table tracks the same state --
 * which buckets' own slots are taken and how many keys hold excess slots -- and refuses exactly then; bulk
 * inserts and erases then run one thread per key under the stripe locks, and a call of at most 4096 keys
 * that could reach the refusal takes its keys in input order, as the reference does on one thread.  Off
 * (on = 0), a table takes keys until no slot is free, through the tile and partitioned kernels.  On by
 * default for tables whose max_size() is at most 2^20; switched only on an empty table (size 0, else
 * SG_ERR_BAD_ARG), starting from the reference's empty state.  Synchronises.  Kept by rehash and clear;
 * the batched tables and the server's tables do not keep it. */
SG_API sg_status sg_unordered_set_excess_accounting(sg_unordered* table, int32_t on, void* stream);
/* Keys holding excess slots (the reference's excess_count minus its free excess slots), -1 with the
 * accounting off.  Synchronises. */
SG_API sg_status sg_unordered_excess_used(sg_unordered* table, void* stream, int64_t* out);

/* A device buffer of at least `bytes` owned by the table, for a caller that stages a bulk call's inputs
 * (the C++ API's custom-key calls turn keys into key words and hashes there): no allocation per call.  Valid
 * until the next call of this function on the table (a larger request replaces the buffer, after a device
 * synchronisation) or the table's destruction; calls on one table are stream-ordered, so one call's staging
 * is not overwritten by the next before it is read.  Allocated with the table's allocator. */
SG_API sg_status sg_unordered_call_scratch(sg_unordered* table, int64_t bytes, void* stream, void** out);

/* erase(begin, end) over keys: src/stdgpu/impl/unordered_base_detail.cuh:1045-1066 (per key :1019-1043).
 * out_erased (nullable): per key 1 if this call erased it, else 0. */
SG_API sg_status sg_unordered_erase(sg_unordered* table, const void* keys, int64_t n, uint8_t* out_erased, void* stream);

/* Bulk form of the device-only find(key): src/stdgpu/impl/unordered_base_detail.cuh:619-682.
 * out_mapped (nullable; maps only): the mapped value of each found key (untouched when absent).
 * out_found (nullable): 1 when the key is present. */
SG_API sg_status sg_unordered_find(sg_unordered* table, const void* keys, int64_t n, void* out_mapped, uint8_t* out_found,
                            void* stream);

/* Bulk form of the device-only contains(key) / count(key): unordered_base_detail.cuh:595-617, 684-706. */
SG_API sg_status sg_unordered_contains(sg_unordered* table, const void* keys, int64_t n, uint8_t* out_flags, void* stream);

/* size(): src/stdgpu/impl/unordered_base_detail.cuh:1121-1132 (synchronises the stream). */
SG_API sg_status sg_unordered_size(sg_unordered* table, void* stream, int64_t* out_size);

/* Device-side conditions the reference only printf()s (unordered_base_detail.cuh:769-772): the number of
 * inserts refused for lack of a free slot since the last call (then reset) and the number of erased slots
 * awaiting reuse.  Returns SG_ERR_FULL when refusals were counted.  Synchronises.  Outputs nullable. */
SG_API sg_status sg_unordered_status(sg_unordered* table, void* stream, int64_t* out_refused, int64_t* out_tombstones);

/* clear(): src/stdgpu/impl/unordered_base_detail.cuh:1220-1252 */
SG_API sg_status sg_unordered_clear(sg_unordered* table, void* stream);

/* valid(): src/stdgpu/impl/unordered_base_detail.cuh:1192-1218 -- the same invariants restated for
 * this layout: every stored key is found at its own slot by its probe sequence (reachable, unique),
 * unused tail slots are untouched, and size() equals the number of stored keys. */
SG_API sg_status sg_unordered_valid(sg_unordered* table, void* stream, int32_t* out_valid);

/* device_range(): src/stdgpu/impl/unordered_base_detail.cuh:160-208.  Writes the slot indices of all
 * stored elements to out_slots (capacity >= max_size() + 2 entries) and their count to *out_n
 * (synchronises).  Element i of the range is ((value_type*)view.slots)[out_slots[i]]. */
SG_API sg_status sg_unordered_device_range(sg_unordered* table, int32_t* out_slots, void* stream, int64_t* out_n);

/* Copy all stored keys (and mapped values for maps; nullable) out, in slot order.  *out_n gets the count. */
SG_API sg_status sg_unordered_range_copy(sg_unordered* table, void* out_keys, void* out_mapped, void* stream,
                                  int64_t* out_n);

/* bucket(key) (host-callable): src/stdgpu/impl/unordered_base_detail.cuh:547-564 -- fibonacci hashing of the
 * identity hash (src/stdgpu/impl/functional_detail.h:60-80).  key points to one key of the table's key type. */
SG_API sg_status sg_unordered_bucket(const sg_unordered* table, const void* key, int64_t* out_bucket);

/* bucket_count(), max_size(), max_load_factor() plus storage facts. */
SG_API sg_status sg_unordered_geometry(const sg_unordered* table, sg_geometry* out);

/* Device view for native device-side find / contains / insert / emplace / erase. */
SG_API sg_status sg_unordered_view_of(const sg_unordered* table, sg_unordered_view* out);

/* Geometry of createDeviceObject(capacity) without creating a table. */
SG_API sg_status sg_unordered_geometry_for(int32_t kind, int64_t capacity, sg_geometry* out);

/* ---------------- table calls on host buffers (no counterpart in the reference) ---------------- */

/* The reference's bulk calls take device iterators; a caller whose keys are in host memory copies them
 * in, calls, and copies the results out.  These entry points take HOST pointers (pinned for overlap)
 * and pipeline the three: the input is cut into chunks of chunk_elems, each copied host->device into one
 * of n_buffers device staging buffers while earlier chunks' kernels run, and each chunk's results are
 * copied device->host while later chunks run.  Every copy of a call starts after the work already on
 * `stream`, and `stream` waits for the call's last result copy, so a call behaves like one
 * stream-ordered operation; host buffers must stay valid until the stream reaches that point.
 * A stager belongs to the device current at its creation and to one host thread at a time; calls on
 * several tables may share it.  Results per element are those of the device-pointer entry points
 * (a duplicate key in one call is inserted once; which copy reports 1 may differ). */
typedef struct sg_stager sg_stager;
/* chunk_elems in [1, 2^30], n_buffers in [2, 8]; holds n_buffers x 33 x chunk_elems device bytes. */
SG_API sg_status sg_stager_create(int64_t chunk_elems, int32_t n_buffers, sg_stager** out);
SG_API sg_status sg_stager_destroy(sg_stager* stager);
/* inputs_ready != 0: a call's host->device copies start when the call is made instead of after the work
 * already queued on the caller's stream (the kernels still run in stream order), so the link keeps busy
 * while earlier calls finish.  The caller vouches that no work queued before a call writes that call's
 * host inputs (for example a download into the same host buffer).  Default 0. */
SG_API sg_status sg_stager_set_inputs_ready(sg_stager* stager, int32_t inputs_ready);
/* sg_unordered_insert / insert_kv / erase / find / contains with host buffers (outputs nullable); the
 * find form writes 0 as the mapped value of an absent key. */
SG_API sg_status sg_unordered_insert_host(sg_unordered* table, sg_stager* stager, const void* values, int64_t n,
                                          uint8_t* out_inserted, void* stream);
SG_API sg_status sg_unordered_insert_kv_host(sg_unordered* table, sg_stager* stager, const void* keys,
                                             const void* mapped, int64_t n, uint8_t* out_inserted, void* stream);
SG_API sg_status sg_unordered_erase_host(sg_unordered* table, sg_stager* stager, const void* keys, int64_t n,
                                         uint8_t* out_erased, void* stream);
SG_API sg_status sg_unordered_find_host(sg_unordered* table, sg_stager* stager, const void* keys, int64_t n,
                                        void* out_mapped, uint8_t* out_found, void* stream);
SG_API sg_status sg_unordered_contains_host(sg_unordered* table, sg_stager* stager, const void* keys, int64_t n,
                                            uint8_t* out_flags, void* stream);

/* ---------------- batched many-table objects (no counterpart in the reference) ---------------- */

/* Thousands of independent unordered_set / unordered_map objects of one kind and uneven capacities,
 * each with the geometry and behaviour of a single table, stored in one device arena.  Every batched
 * operation takes the keys of all tables concatenated, table t owning elements [offsets[t],
 * offsets[t+1]) of the input (offsets: DEVICE array of n_tables + 1 int64), and runs as one
 * persistent launch over (table, 32-key range) tiles.  A NULL key array (all ranges empty, as an empty
 * tensor gives) walks no tile.  No host work depends on the sizes, so a sequence of batched calls can be
 * captured in a CUDA graph. */
typedef struct sg_table_batch sg_table_batch;

/* capacities: HOST array of n_tables capacities (createDeviceObject(capacity) of each table). */
SG_API sg_status sg_batch_create(int32_t kind, int32_t n_tables, const int64_t* capacities, void* stream,
                                 sg_table_batch** out);
SG_API sg_status sg_batch_destroy(sg_table_batch* batch);
/* Launch shape of the walking kernels: threads per block (128, 256, 512), resident blocks per SM
 * (0 = as many as fit), tiles each warp takes per step (1..64). */
SG_API sg_status sg_batch_configure(sg_table_batch* batch, int32_t threads_per_block, int32_t blocks_per_sm,
                                    int32_t tiles_per_step);
/* clear() of every table */
SG_API sg_status sg_batch_clear(sg_table_batch* batch, void* stream);
/* insert(begin, end) per table over value_type elements / over keys and mapped values */
SG_API sg_status sg_batch_insert(sg_table_batch* batch, const void* values, const int64_t* offsets,
                                 uint8_t* out_inserted, void* stream);
SG_API sg_status sg_batch_insert_kv(sg_table_batch* batch, const void* keys, const void* mapped,
                                    const int64_t* offsets, uint8_t* out_inserted, void* stream);
SG_API sg_status sg_batch_erase(sg_table_batch* batch, const void* keys, const int64_t* offsets,
                                uint8_t* out_erased, void* stream);
SG_API sg_status sg_batch_find(sg_table_batch* batch, const void* keys, const int64_t* offsets, void* out_mapped,
                               uint8_t* out_found, void* stream);
SG_API sg_status sg_batch_contains(sg_table_batch* batch, const void* keys, const int64_t* offsets,
                                   uint8_t* out_flags, void* stream);
/* size() of every table into a HOST array of n_tables (synchronises). */
SG_API sg_status sg_batch_sizes(sg_table_batch* batch, void* stream, int64_t* out_sizes);
/* Device view of table t for native device calls. */
SG_API sg_status sg_batch_view_of(const sg_table_batch* batch, int32_t table, sg_unordered_view* out);
SG_API sg_status sg_batch_info(const sg_table_batch* batch, int64_t* out_storage_bytes, int32_t* out_n_tables);

/* ---------------- served request stream (no counterpart in the reference) ---------------- */

/* A scheduler thread keeps tables of one kind resident and executes submitted requests with
 * continuous batching: whenever launches complete or requests arrive, every table with pending requests
 * and nothing in flight contributes its run of consecutive same-operation requests.  Small runs of one
 * operation share one segmented launch on a high-priority stream; a run of many keys (sg_server_set_policy)
 * runs as its own launches, cut into chunks, on a low-priority stream, with a cap on how many such runs
 * are in flight, so small requests of other tables are not held behind it.  Each launch completes its own
 * requests.  Requests on one table execute in submission order.  Tables are admitted, and grown (rehashed
 * into a table of the next doubling of the capacity that holds the run, on the device with no host round
 * trip, while the table's later requests wait) before an insert run would pass 85 % of max_size(), only
 * while the HBM budget allows; otherwise the table admission or the request is refused with SG_ERR_BUDGET
 * -- nothing spills to host memory.  The storage a grow replaced counts against the budget until the
 * server is next idle (or the budget needs it).  Table storage comes from a stream-ordered memory pool the
 * server owns, into which a quarter of the budget is mapped at creation: what the pool releases stays mapped
 * for later tables until the server is destroyed, so the device memory the process holds is the larger of
 * that quarter and the largest total the tables reached, and a grow rarely has to map new memory.
 * Within one run of same-operation requests the per-key inserted / erased flags of a key repeated in
 * several requests may fall on any of them (as for duplicates within one bulk call). */
typedef struct sg_server sg_server;

typedef enum sg_server_op
{
    SG_SERVER_INSERT = 0,
    SG_SERVER_FIND = 1,
    SG_SERVER_ERASE = 2
} sg_server_op;

typedef struct sg_request
{
    int32_t table;      /* table id given to sg_server_admit_table */
    int32_t op;         /* sg_server_op */
    int64_t n;          /* keys */
    const void* keys;   /* DEVICE, n keys; must stay valid until the request completes */
    const void* mapped; /* DEVICE, n mapped values for inserts into maps (nullable) */
    void* out_mapped;   /* DEVICE, n mapped values written by finds on maps (nullable) */
    uint8_t* out_flags; /* DEVICE, n flags: inserted / found / erased (nullable) */
} sg_request;

typedef struct sg_server_stats
{
    int64_t requests_done;
    int64_t keys_done;
    double p50_us;     /* request latency, submission to completion */
    double p99_us;
    double max_us;
    double keys_per_s; /* keys of completed requests over first submission .. last completion */
    int64_t launches;
    int64_t waves;
    int64_t refused_budget;
    int64_t rehashes;
    int64_t hbm_used_bytes;
    double grow_host_us;     /* scheduler time spent launching grows (allocation of the new table included) */
    double max_grow_host_us; /* the longest of them */
    double grow_create_us;   /* the grow thread's time creating the grown tables (their allocation included) */
} sg_server_stats;

SG_API sg_status sg_server_create(int32_t kind, int64_t hbm_budget_bytes, int32_t n_streams, int32_t n_slots,
                                  sg_server** out);
/* Waits for requests in flight, then frees every table. */
SG_API sg_status sg_server_destroy(sg_server* server);
/* createDeviceObject(capacity) for table id `table`, if the budget allows (else SG_ERR_BUDGET). */
SG_API sg_status sg_server_admit_table(sg_server* server, int32_t table, int64_t capacity);
/* Waits for the table's requests, then destroyDeviceObject. */
SG_API sg_status sg_server_drop_table(sg_server* server, int32_t table);
/* Non-blocking; returns a ticket. */
SG_API sg_status sg_server_submit(sg_server* server, const sg_request* request, int64_t* out_ticket);
/* Submits n requests in order in one call (one ticket each). */
SG_API sg_status sg_server_submit_many(sg_server* server, const sg_request* requests, int32_t n, int64_t* out_tickets);
/* While paused, submitted requests queue and no new launch starts (launches in flight finish);
 * resuming lets the queued requests coalesce into the next waves. */
SG_API sg_status sg_server_set_paused(sg_server* server, int32_t paused);
/* Request-size policy: a table's run of same-operation requests with at least direct_keys keys runs as
 * its own launches of at most chunk_keys keys each on one of direct_streams (1..n_streams) low-priority
 * streams, with at most max_direct (1..16) such runs issued and not complete; defaults 65536, 4194304, 8
 * and 4. */
SG_API sg_status sg_server_set_policy(sg_server* server, int64_t direct_keys, int64_t chunk_keys, int32_t max_direct,
                                      int32_t direct_streams);
/* Growing ahead (default on): a table that an insert or erase run left more than half full, with no request
 * waiting, grows to the next doubling of its capacity while it is idle, within the budget as it stands, so a
 * later insert does not wait for the rehash. */
SG_API sg_status sg_server_set_grow_ahead(sg_server* server, int32_t enabled);
/* Waits (timeout_ms < 0: no limit) for a ticket; out_request_status: SG_OK or SG_ERR_BUDGET (refused). */
SG_API sg_status sg_server_wait(sg_server* server, int64_t ticket, int32_t timeout_ms, sg_status* out_request_status);
/* Waits for every submitted request. */
SG_API sg_status sg_server_drain(sg_server* server, int32_t timeout_ms);
SG_API sg_status sg_server_get_stats(sg_server* server, sg_server_stats* out);
/* Latency of a completed request (submission to completion, microseconds); SG_ERR_BAD_ARG for an unknown
 * ticket, SG_ERR_RETRY_EXHAUSTED while it is not complete. */
SG_API sg_status sg_server_request_latency(sg_server* server, int64_t ticket, double* out_us);
/* Waits for the table's requests, then size(). */
SG_API sg_status sg_server_table_size(sg_server* server, int32_t table, int64_t* out_size);
/* Waits for the table's requests (and a grow in flight), then its device view. */
SG_API sg_status sg_server_table_view(sg_server* server, int32_t table, sg_unordered_view* out);

/* ---------------- vector<T> (T = 4 or 8 bytes) ---------------- */

typedef struct sg_vector sg_vector;

typedef struct sg_vector_view
{
    void* data;
    void* size; /* device int64 counter; may exceed capacity transiently, size() clamps (vector_detail.cuh:484-511) */
    int64_t capacity;
    int32_t elem_bytes;
    int32_t pad;
    void* slot_state; /* device, one 16-bit word per element: (epoch << 1) | occupied, written by device calls */
    void* sync;       /* device: the epoch of the last bulk call and the size it left (sg_vector_sync) */
} sg_vector_view;

/* Device-call state of a vector.  Device push_back and pop_back may share a launch: each takes its position
 * from the counter, then waits (bounded) until its slot is free (push) or written (pop), as the reference's
 * per-slot occupied bit and lock do (vector_detail.cuh:181-299).  A slot word whose epoch is not the
 * current one has not been touched since the last bulk call and reads as occupied exactly when its index
 * is below base_size, so bulk calls never touch the slot words: each ends by advancing the epoch. */
typedef struct sg_vector_sync
{
    uint32_t epoch;     /* 1 .. 32767 */
    uint32_t error;     /* bit 0: a device wait gave up */
    int64_t base_size;  /* size() after the last bulk call */
} sg_vector_sync;

/* vector::createDeviceObject(capacity): src/stdgpu/impl/vector_detail.cuh (createDeviceObject) */
SG_API sg_status sg_vector_create(int32_t elem_bytes, int64_t capacity, sg_vector** out);
/* createDeviceObject(capacity, allocator): sg_vector_create with every device block of the object taken from
 * `allocator` (sg_allocator; copied; alloc and release non-null, release_ctx called at destroy). */
SG_API sg_status sg_vector_create_with_allocator(int32_t elem_bytes, int64_t capacity, const sg_allocator* allocator,
                                       sg_vector** out);
SG_API sg_status sg_vector_destroy(sg_vector* vec);
/* Bulk form of the device push_back (src/stdgpu/impl/vector_detail.cuh:181-238): element i is pushed when
 * pred == NULL or pred[i] != 0.  out_pushed (nullable) gets 1 for each element that was stored. */
SG_API sg_status sg_vector_push_back(sg_vector* vec, const void* values, const uint8_t* pred, int64_t n,
                              uint8_t* out_pushed, void* stream);
/* size() (clamped to [0, capacity]): src/stdgpu/impl/vector_detail.cuh:484-511 */
SG_API sg_status sg_vector_size(sg_vector* vec, void* stream, int64_t* out_size);
/* clear() */
SG_API sg_status sg_vector_clear(sg_vector* vec, void* stream);
/* pop_back() n times (src/stdgpu/impl/vector_detail.cuh:240-299): element i takes the i-th element from the
 * back; out_ok[i] = 0 once the vector is empty.  Outputs nullable. */
SG_API sg_status sg_vector_pop_back(sg_vector* vec, int64_t n, void* out_values, uint8_t* out_ok, void* stream);
/* insert(device_end(), begin, end) (vector_detail.cuh:372-410): appends n device values; SG_ERR_FULL and
 * nothing inserted when they do not fit.  Synchronises. */
SG_API sg_status sg_vector_insert(sg_vector* vec, const void* values, int64_t n, void* stream);
/* erase(device_end() - n, device_end()) (vector_detail.cuh:418-450): drops the last n elements;
 * SG_ERR_BAD_ARG and nothing erased when n > size().  Synchronises. */
SG_API sg_status sg_vector_erase(sg_vector* vec, int64_t n, void* stream);
SG_API sg_status sg_vector_view_of(const sg_vector* vec, sg_vector_view* out);

/* ---------------- deque<T> (T = 4 or 8 bytes), push_back / pop_front ---------------- */

typedef struct sg_deque sg_deque;

typedef struct sg_deque_view
{
    void* data;
    void* seq;      /* per-slot turn counter of the ring (uint32) */
    void* counters; /* device {int64 size, uint64 begin, uint64 end, uint32 error, uint32 pad, int64 avail,
                     * uint64 op_t0, int64 op_k}; begin / end are tickets, ticket mod capacity is the slot */
    int64_t capacity;
    int32_t elem_bytes;
    int32_t pad;
    void* slot_state; /* device, one 16-bit word per slot: (epoch << 1) | occupied, written by device calls */
    void* sync;       /* device sg_deque_sync */
} sg_deque_view;

/* Device-call state of a deque.  The device calls (push_back, push_front, pop_front, pop_back, in any mix
 * in one launch) take their ticket from the counters and then wait (bounded) on the slot's word until the
 * slot is free (push) or written (pop), the reference's per-slot occupied bit
 * (src/stdgpu/impl/deque_detail.cuh:202-446).  A word of another epoch has not been touched since the last
 * bulk call: its slot is occupied exactly when its ticket lay in [base_begin, base_end) after that call.
 * Device calls set `dirty`; the next bulk call first rebuilds the turn words its own kernels wait on. */
typedef struct sg_deque_sync
{
    uint32_t epoch; /* 1 .. 32767 */
    uint32_t dirty;
    uint64_t base_begin;
    uint64_t base_end;
} sg_deque_sync;

/* deque::createDeviceObject(capacity): src/stdgpu/impl/deque_detail.cuh (createDeviceObject) */
SG_API sg_status sg_deque_create(int32_t elem_bytes, int64_t capacity, sg_deque** out);
/* createDeviceObject(capacity, allocator): sg_deque_create with every device block of the object taken from
 * `allocator` (sg_allocator; copied; alloc and release non-null, release_ctx called at destroy). */
SG_API sg_status sg_deque_create_with_allocator(int32_t elem_bytes, int64_t capacity, const sg_allocator* allocator,
                                       sg_deque** out);
SG_API sg_status sg_deque_destroy(sg_deque* dq);
/* Mixed launch: element i does push_back(values[i]) when is_push[i] != 0, else pop_front().
 * deque_detail.cuh:202-258 (push_back) and :388-446 (pop_front).  out_popped / out_ok nullable.
 * is_push == NULL means all push_back. */
SG_API sg_status sg_deque_ops(sg_deque* dq, const uint8_t* is_push, const void* values, int64_t n, void* out_popped,
                       uint8_t* out_ok, void* stream);
/* size() (clamped): src/stdgpu/impl/deque_detail.cuh:486-520; SG_ERR_RETRY_EXHAUSTED if a wait gave up */
SG_API sg_status sg_deque_size(sg_deque* dq, void* stream, int64_t* out_size);
/* Copy the stored elements front to back to out (device) and return their count (synchronises). */
SG_API sg_status sg_deque_copy_out(sg_deque* dq, void* out, void* stream, int64_t* out_n);
SG_API sg_status sg_deque_clear(sg_deque* dq, void* stream);
/* push_front() / pop_back() n times (deque_detail.cuh:314-386, :260-312), one kind per launch: element i acts
 * as the i-th of a sequence of calls (push_front of values[0..n) leaves values[n-1] at the front; pop_back
 * pops the back element first).  Launches of either kind may follow sg_deque_ops launches on the same stream
 * in any order.  out_ok / out_popped nullable. */
SG_API sg_status sg_deque_push_front(sg_deque* dq, const void* values, int64_t n, uint8_t* out_ok, void* stream);
SG_API sg_status sg_deque_pop_back(sg_deque* dq, int64_t n, void* out_popped, uint8_t* out_ok, void* stream);
SG_API sg_status sg_deque_view_of(const sg_deque* dq, sg_deque_view* out);

/* ---------------- bitset<unsigned int>::count ---------------- */

/* bitset::count(): src/stdgpu/impl/bitset_detail.cuh:388-404 with count_block_bits :130-160.
 * blocks: ceil(nbits / 32) 32-bit blocks, bit i = bit (i % 32) of blocks[i / 32]; bits at or above
 * nbits in the last block are masked off.  Synchronises and returns the count. */
SG_API sg_status sg_bitset_count(const uint32_t* blocks, int64_t nbits, void* stream, int64_t* out_count);

/* Allocation-free form of sg_bitset_count.  It has no counterpart in the reference.
 * For callers that must not allocate device memory: processes whose device memory is owned by another
 * allocator with a budget fixed up front (a framework's pool that leaves nothing for a library to
 * cudaMalloc), and latency-critical paths that cannot take the device-wide synchronisation that
 * cudaMalloc / cudaFree imply.  sg_bitset_count allocates its per-block partial sums on first use; this entry point
 * keeps them in a fixed array compiled into the library instead (64 KiB, present on every GPU that
 * loads the library until the process exits) and calls no allocator.  The count is written to
 * out_count, which is DEVICE memory owned by the caller; the call is asynchronous on `stream`.
 * Limit: nbits <= 2^34 (2 GiB of blocks); larger inputs return SG_ERR_BAD_ARG.  All calls on a device
 * share the array, so two calls whose kernels overlap on the GPU (unordered streams) race and give
 * wrong counts: order them on one stream or with events.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress); make that first call before any stream capture.  The
 * address is kept for the life of the process: after a cudaDeviceReset of that device (which also ends
 * every other allocation of this library there) the entry point must not be called again. */
SG_API sg_status sg_bitset_count_noalloc(const uint32_t* blocks, int64_t nbits, int64_t* out_count, void* stream);

/* ---------------- library ---------------- */

/* Random-read ceiling of the device memory (a diagnostic with no counterpart in the reference): `reads`
 * reads of unit_bytes (32, 64 or 128) each at random positions of a freshly allocated device buffer of
 * buffer_bytes (>= 1 MiB; make it far larger than L2), timed with events on `stream` (best of three after
 * a warm-up); the rate in reads per second goes to out_reads_per_s.  The table kernels read one random
 * 128-byte group line per key, so this rate bounds them alongside the copy bandwidth.  Synchronises. */
SG_API sg_status sg_measure_random_reads(int64_t buffer_bytes, int64_t reads, int32_t unit_bytes, void* stream,
                                         double* out_reads_per_s);

/* Number of kernels this library has launched since load (all entry points). */
SG_API int64_t sg_kernel_launch_count(void);
/* Human-readable text for a status. */
SG_API const char* sg_status_string(sg_status status);

#ifdef __cplusplus
}
#endif

#endif /* STDGPU_GB300_H */
