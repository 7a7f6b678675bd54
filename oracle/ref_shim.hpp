// ref_shim.hpp -- lets the reference's OpenCL C kernel source compile as C++20
// so that its own kernels can run on the host as a second oracle leg and as the
// timed CPU baseline.  TEST INFRASTRUCTURE ONLY (see oracle/m2_oracle.c).
//
// OpenCL address-space qualifiers become empty, work-item queries read a
// per-thread index set by the driver loop (one kernel "launch" = a loop over
// its global ids), and the few OpenCL built-ins the source uses (clz, min,
// uchar2/ulong2) get C++ definitions.  barrier() is a no-op: only kernels that
// do not use __local memory are ever driven (M2's generic plan).
#pragma once
#include <cstddef>
#include <cstdint>
#include <sys/types.h>

#define __kernel
#define __global
#define __local
#define __private
#define __constant const
#define restrict __restrict__
#define inline inline
#define CLK_LOCAL_MEM_FENCE 0
#define CLK_GLOBAL_MEM_FENCE 0

typedef unsigned char uchar;
typedef unsigned short ushort;
struct uchar2 { uchar s0, s1; };
struct ulong2 { ulong s0, s1; };

namespace refshim {
extern thread_local size_t gid;
}
static inline size_t get_global_id(int) { return refshim::gid; }
static inline size_t get_local_id(int) { return 0; }
static inline size_t get_group_id(int) { return refshim::gid; }
static inline size_t get_local_size(int) { return 1; }
static inline void barrier(int) {}
// OpenCL clz(0) is the bit width; __builtin_clz(0) is undefined.
static inline uint clz(uint x) { return x ? (uint)__builtin_clz(x) : 32u; }
template <class A, class B> static inline auto min(A a, B b) { return a < b ? a : b; }
