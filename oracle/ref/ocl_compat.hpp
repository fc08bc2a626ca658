/*
 * ocl_compat.hpp -- lets the reference's OpenCL C kernels for the CPU
 * (opencl/pp/pp_common.cl + opencl/pp/pp_cpu.cl of nunofachada/pphpc)
 * compile UNMODIFIED as C++ for the host, so that the reference's own CPU
 * algorithm can run here as a checker and a CPU baseline.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle/ref/build_ref.py): nothing in the
 * product includes this file.
 *
 * What an OpenCL C compiler and runtime provide, restated for a host:
 *   - the address-space and kernel qualifiers (__kernel, __global,
 *     __private) vanish: host memory is one address space;
 *   - uint / ushort / uchar / ulong are the fixed-width unsigned types;
 *     `uint` is a thin class so that its shifts follow OpenCL C, where the
 *     shift count is taken modulo the operand's width (OpenCL C 1.2,
 *     section 6.3 j): pp_cpu.cl:218 shifts a uint right by 35, which OpenCL
 *     defines as a shift by 3 and C++ leaves undefined;
 *   - get_global_id(0) / get_global_size(0) read the work-item identity the
 *     host loop sets for the calling thread;
 *   - atomic_add / atomic_cmpxchg on 32-bit words map to the GCC __atomic
 *     builtins (relaxed order, as OpenCL 1.x atomics);
 *   - min() as in OpenCL C for unsigned operands;
 *   - the compile-time model constants the reference passes with -D
 *     (pp_cpu.c:801-852) are globals set per run by the host loop, except
 *     MAX_AGENT_SHUF, which the kernel tests with #if and so stays a
 *     compile-time constant (the reference's default, 256);
 *   - clo_statetype / clo_rng_next / clo_rng_next_int stand for the RNG of
 *     cl_ops, a third-party library (unpinned version) absent from the
 *     reference tree. Each work item owns one 64-bit state in seeds[gid];
 *     clo_rng_next advances it with xorshift64* (S. Vigna, "An experimental
 *     exploration of Marsaglia's xorshift generators, scrambled", ACM TOMS
 *     42(4), 2016) and returns the high 32 bits; clo_rng_next_int(seeds, n)
 *     maps such a word to [0, n) by the multiply-shift floor(w * n / 2^32).
 *     The reference's draws are therefore not reproduced bit for bit; its
 *     algorithm (what is drawn, when, by which work item) is.
 *
 * This header includes no system header, so the preprocessed kernel
 * translation unit (compat + the reference's kernels) compiles unchanged on
 * any LP64 host.
 */
#ifndef OCL_COMPAT_HPP
#define OCL_COMPAT_HPP

#define __kernel
#define __global
#define __private
#define UINT_MAX 0xffffffffu

typedef unsigned short ushort;
typedef unsigned char uchar;
typedef unsigned long ulong;

namespace ocl {

/* OpenCL C's 32-bit unsigned int: arithmetic through the built-in unsigned
 * type, shifts with the count taken modulo 32. Trivial, so it may sit in a
 * union (pp_cpu.cl:78-84). */
struct uint_t {
	unsigned v;
	uint_t() = default;
	constexpr uint_t(unsigned x) : v(x) {}
	constexpr operator unsigned() const { return v; }
	uint_t &operator+=(unsigned o) { v += o; return *this; }
	uint_t &operator-=(unsigned o) { v -= o; return *this; }
	uint_t &operator^=(unsigned o) { v ^= o; return *this; }
	uint_t &operator|=(unsigned o) { v |= o; return *this; }
	uint_t &operator&=(unsigned o) { v &= o; return *this; }
	uint_t &operator++() { ++v; return *this; }
	uint_t &operator--() { --v; return *this; }
	uint_t operator++(int) { uint_t o = *this; ++v; return o; }
	uint_t operator--(int) { uint_t o = *this; --v; return o; }
};
inline unsigned operator<<(uint_t a, int s) { return a.v << (s & 31); }
inline unsigned operator>>(uint_t a, int s) { return a.v >> (s & 31); }

/* Work-item identity of the calling host thread (set by the host loop). */
extern thread_local unsigned long tl_gid, tl_gws;

/* Model constants of the current run (the reference's -D options). */
extern unsigned max_agents, rows_per_workitem;
extern unsigned init_sheep, sheep_gain, sheep_thr, sheep_prob;
extern unsigned init_wolves, wolves_gain, wolves_thr, wolves_prob;
extern unsigned grass_restart, grid_x, grid_y, iters;

inline unsigned long get_global_id(int) { return tl_gid; }
inline unsigned long get_global_size(int) { return tl_gws; }

inline unsigned atomic_add(uint_t *p, unsigned x)
{
	return __atomic_fetch_add(&p->v, x, __ATOMIC_RELAXED);
}

inline unsigned atomic_cmpxchg(uint_t *p, unsigned cmp, unsigned val)
{
	unsigned expected = cmp;
	__atomic_compare_exchange_n(&p->v, &expected, val, false,
		__ATOMIC_RELAXED, __ATOMIC_RELAXED);
	return expected;
}

inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }

typedef unsigned long long clo_statetype;

inline unsigned clo_rng_next(clo_statetype *seeds, unsigned long gid)
{
	unsigned long long x = seeds[gid];
	x ^= x >> 12;
	x ^= x << 25;
	x ^= x >> 27;
	seeds[gid] = x;
	return (unsigned) ((x * 0x2545F4914F6CDD1DULL) >> 32);
}

inline unsigned clo_rng_next_int(clo_statetype *seeds, unsigned n)
{
	return (unsigned) (((unsigned long long) clo_rng_next(seeds, tl_gid) * n) >> 32);
}

} /* namespace ocl */

#define MAX_AGENTS ::ocl::max_agents
#define ROWS_PER_WORKITEM ::ocl::rows_per_workitem
#define INIT_SHEEP ::ocl::init_sheep
#define SHEEP_GAIN_FROM_FOOD ::ocl::sheep_gain
#define SHEEP_REPRODUCE_THRESHOLD ::ocl::sheep_thr
#define SHEEP_REPRODUCE_PROB ::ocl::sheep_prob
#define INIT_WOLVES ::ocl::init_wolves
#define WOLVES_GAIN_FROM_FOOD ::ocl::wolves_gain
#define WOLVES_REPRODUCE_THRESHOLD ::ocl::wolves_thr
#define WOLVES_REPRODUCE_PROB ::ocl::wolves_prob
#define GRASS_RESTART ::ocl::grass_restart
#define GRID_X ::ocl::grid_x
#define GRID_Y ::ocl::grid_y
#define ITERS ::ocl::iters
#ifndef MAX_AGENT_SHUF
#define MAX_AGENT_SHUF 256
#endif

#endif
