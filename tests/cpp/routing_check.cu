// Compile-time check of which storage each element type takes in the C++ API (include/stdgpu_gb300/stdgpu.cuh):
// integer keys with the default hash and integer mapped values -> the library's precompiled kinds; other
// trivially copyable keys of at most 8 bytes with a 4/8-byte trivially copyable mapped type -> the word-keyed
// custom path; everything else -> the wide tables, and so do keys compared by a user KeyEqual or whose bytes do
// not decide equality (floating point, padding).  Builds to a program that does nothing.
#include <cstdio>
#include <cstdint>
#include <type_traits>

#include <stdgpu_gb300/stdgpu.cuh>

struct short3_key
{
    std::int16_t x, y, z;
};
struct vec3i32_key
{
    std::int32_t x, y, z;
};
struct key16
{
    std::uint64_t a, b;
};
struct with_destructor
{
    std::uint32_t v = 0;
    __host__ __device__ ~with_destructor() {}
};
struct empty_tag
{
};
struct any_hash
{
    template <typename K>
    __host__ __device__ std::size_t
    operator()(const K&) const
    {
        return 0;
    }
};

template <typename Container, typename Base>
constexpr bool routes_to = std::is_base_of<Base, Container>::value;

using namespace stdgpu;
using detail::custom_map;
using detail::custom_set;
using detail::native_map;
using detail::native_set;
using detail::wide_map;
using detail::wide_set;

// precompiled kinds
using m1 = unordered_map<std::uint64_t, std::uint32_t>;
using m2 = unordered_map<std::uint32_t, std::uint64_t>;
using s1 = unordered_set<std::uint32_t>;
static_assert(routes_to<m1, native_map<std::uint64_t, std::uint32_t, m1>>, "u64 -> u32 map");
static_assert(routes_to<m2, native_map<std::uint32_t, std::uint64_t, m2>>, "u32 -> u64 map");
static_assert(routes_to<s1, native_set<std::uint32_t, s1>>, "u32 set");

// word-keyed custom path
using c1 = unordered_set<short3_key, any_hash>;
using c2 = unordered_map<short3_key, float, any_hash>;
using c3 = unordered_map<std::uint64_t, float>; // integer key, non-integer mapped type
using c4 = unordered_map<std::uint64_t, std::uint32_t, any_hash>; // integer key, user hash
static_assert(routes_to<c1, custom_set<short3_key, any_hash, c1>>, "6-byte key set");
static_assert(routes_to<c2, custom_map<short3_key, float, any_hash, c2>>, "6-byte key, float");
static_assert(routes_to<c3, custom_map<std::uint64_t, float, hash<std::uint64_t>, c3>>, "u64 -> float");
static_assert(routes_to<c4, custom_map<std::uint64_t, std::uint32_t, any_hash, c4>>, "u64 with a user hash");

// wide tables
using w1 = unordered_set<vec3i32_key, any_hash>;
using w2 = unordered_map<key16, std::uint64_t, any_hash>;
using w3 = unordered_map<std::uint64_t, key16>;
using w4 = unordered_map<std::uint32_t, with_destructor>;
using w5 = unordered_map<vec3i32_key, empty_tag, any_hash>;
using w6 = unordered_set<with_destructor, any_hash>;
static_assert(routes_to<w1, wide_set<vec3i32_key, any_hash, w1>>, "12-byte key set");
static_assert(routes_to<w2, wide_map<key16, std::uint64_t, any_hash, w2>>, "16-byte key");
static_assert(routes_to<w3, wide_map<std::uint64_t, key16, hash<std::uint64_t>, w3>>, "16-byte mapped type");
static_assert(routes_to<w4, wide_map<std::uint32_t, with_destructor, hash<std::uint32_t>, w4>>,
              "mapped type with a destructor");
static_assert(routes_to<w5, wide_map<vec3i32_key, empty_tag, any_hash, w5>>, "empty mapped type");
// a key that is not trivially copyable compares through its KeyEqual
static_assert(routes_to<w6, wide_set<with_destructor, any_hash, w6, equal_to<with_destructor>>>,
              "key with a destructor");

// keys whose bytes do not decide equality, or a user KeyEqual: the wide tables, comparing with KeyEqual
struct x_only_equal
{
    template <typename K>
    __host__ __device__ bool
    operator()(const K& a, const K& b) const
    {
        return a.x == b.x;
    }
};
struct padded_key
{
    std::uint32_t x;
    std::uint16_t y; // two bytes of padding follow
};
using e1 = unordered_set<short3_key, any_hash, x_only_equal>;
using e2 = unordered_map<float, std::uint32_t, any_hash>;
using e3 = unordered_map<padded_key, std::uint64_t, any_hash>;
using e4 = unordered_set<std::uint64_t, hash<std::uint64_t>, std::equal_to<std::uint64_t>>;
using e5 = unordered_set<std::uint64_t, hash<std::uint64_t>, equal_to<>>;
static_assert(routes_to<e1, wide_set<short3_key, any_hash, e1, x_only_equal>>, "user KeyEqual");
static_assert(routes_to<e2, wide_map<float, std::uint32_t, any_hash, e2, equal_to<float>>>, "floating-point key");
static_assert(routes_to<e3, wide_map<padded_key, std::uint64_t, any_hash, e3, equal_to<padded_key>>>,
              "key with padding");
static_assert(routes_to<e4, native_set<std::uint64_t, e4>>, "std::equal_to on an integer key compares bytes");
static_assert(routes_to<e5, native_set<std::uint64_t, e5>>, "equal_to<void> on an integer key compares bytes");

// the allocator parameter and get_allocator()
using a1 = unordered_map<std::uint64_t, std::uint32_t, hash<std::uint64_t>, equal_to<std::uint64_t>,
                         safe_device_allocator<pair<const std::uint64_t, std::uint32_t>>>;
static_assert(std::is_same<a1, m1>::value, "the default allocator is the reference's");
static_assert(std::is_same<decltype(a1{}.get_allocator()), safe_device_allocator<pair<const std::uint64_t, std::uint32_t>>>::value,
              "get_allocator() returns the allocator type");

int
main()
{
    std::setvbuf(stdout, nullptr, _IOLBF, 0); // each line out before a failure can end the program
    return 0;
}
