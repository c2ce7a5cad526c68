// Force-included (-include) when the reference's own translation units are
// compiled as the pinning oracle.  Maps the MSVC-only spellings they use onto
// GCC equivalents.  Test infrastructure only.
#pragma once
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <cmath>
#include <cassert>
#include <functional>
#include <atomic>
#include <mutex>
#include <condition_variable>
#define __forceinline inline __attribute__((always_inline))
#define __declspec(x)
// WorldOctreeNode.hpp calls the MSVC-internal std::hash<uint32_t>::_Do_hash;
// libstdc++ exposes the nested result_type, which turns the call into a
// functional cast of the 32-bit code (the hash value itself is not used on the
// extraction path).
#define _Do_hash result_type
static inline void* _aligned_malloc(size_t size, size_t align) {
  size_t rounded = (size + align - 1) / align * align;
  return std::aligned_alloc(align, rounded ? rounded : align);
}
static inline void _aligned_free(void* p) { std::free(p); }
