/*
 * Oracle restatement (test infrastructure only, never linked into the product).
 *
 * A sequential plain-C restatement of the reference's hashed-container
 * algorithm (stdgpu 1.3.0, src/stdgpu/impl/unordered_base*.cuh) and of the
 * vector / deque / bitset operations on the same path.  Run sequentially, the
 * reference's lock-and-retry protocol reduces to the plain steps written here;
 * every function names the reference lines it follows.  It is pinned against
 * fixtures produced by the reference library itself (tests/golden/).
 *
 * Keys are carried as uint64_t (the reference's hash<uint32_t> and
 * hash<uint64_t> are both the identity cast to size_t, so a 32-bit key and its
 * zero extension hash identically); values are carried as uint64_t.
 */
#ifndef SG_ORACLE_PORT_H
#define SG_ORACLE_PORT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct port_table port_table;

/* geometry of createDeviceObject(capacity): unordered_base_detail.cuh:1264-1273 */
void port_geometry(int64_t capacity, int64_t* bucket_count, int64_t* excess_count, int64_t* total_count);
/* fibonacci_hashing: unordered_base_detail.cuh:56-85 */
int64_t port_fibonacci_hashing(uint64_t hash, int64_t bucket_count);
/* expected_collisions: unordered_base_detail.cuh:34-48 */
int64_t port_expected_collisions(int64_t bucket_count, int64_t capacity);

port_table* port_create(int64_t capacity);
void port_destroy(port_table* t);
/* per-key device insert / erase (returns 1 on success) */
int port_insert(port_table* t, uint64_t key, uint64_t value);
int port_erase(port_table* t, uint64_t key);
/* find: returns 1 and writes *value when present */
int port_find(const port_table* t, uint64_t key, uint64_t* value);
/* bulk forms over arrays, applied in index order; flags may be NULL */
void port_insert_bulk(port_table* t, const uint64_t* keys, const uint64_t* values, int64_t n, uint8_t* flags);
void port_erase_bulk(port_table* t, const uint64_t* keys, int64_t n, uint8_t* flags);
void port_find_bulk(const port_table* t, const uint64_t* keys, int64_t n, uint64_t* values, uint8_t* found);
/* the same with a caller-supplied Hash(key) per key (custom key types; bucket = fibonacci_hashing(hash)) */
int port_insert_h(port_table* t, uint64_t key, uint64_t hash, uint64_t value);
int port_erase_h(port_table* t, uint64_t key, uint64_t hash);
int port_find_h(const port_table* t, uint64_t key, uint64_t hash, uint64_t* value);
void port_insert_bulk_h(port_table* t, const uint64_t* keys, const uint64_t* hashes, const uint64_t* values, int64_t n,
                        uint8_t* flags);
void port_erase_bulk_h(port_table* t, const uint64_t* keys, const uint64_t* hashes, int64_t n, uint8_t* flags);
void port_find_bulk_h(const port_table* t, const uint64_t* keys, const uint64_t* hashes, int64_t n, uint64_t* values,
                      uint8_t* found);
int64_t port_size(const port_table* t);
int64_t port_bucket_count(const port_table* t);
int64_t port_max_size(const port_table* t);
int64_t port_excess_used(const port_table* t);
int64_t port_bucket(const port_table* t, uint64_t key);
int64_t port_bucket_size(const port_table* t, int64_t n);
void port_clear(port_table* t);
int port_valid(const port_table* t);
/* occupied entries in slot order; returns their count */
int64_t port_range(const port_table* t, uint64_t* keys, uint64_t* values);

/* vector<T>::push_back applied in index order (vector_detail.cuh:181-238);
 * returns size() afterwards, contents to out (storage order). */
int64_t port_vector_push_back(int64_t capacity, const uint64_t* values, const uint8_t* pred, int64_t n,
                              uint8_t* pushed, uint64_t* out);
/* deque<T>: n_init push_backs then ops in index order; op[i]: 0 pop_front (deque_detail.cuh:388-446),
 * 1 push_back (:202-258), 2 push_front (:314-386), 3 pop_back (:260-312) */
int64_t port_deque_ops(int64_t capacity, const uint64_t* init, int64_t n_init, const uint8_t* is_push,
                       const uint64_t* values, int64_t n, uint64_t* popped, uint8_t* ok, uint64_t* remaining);
/* bitset<unsigned int>::count over nbits bits (bitset_detail.cuh:130-160, 388-404) */
int64_t port_bitset_count(const uint32_t* words, int64_t nbits);

#ifdef __cplusplus
}
#endif

#endif
