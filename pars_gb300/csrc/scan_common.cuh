// scan_common.cuh — helpers shared by the scan kernels (scan_ws.cu, scan.cu).
#pragma once

#include <cstdint>

#include "device.cuh"

namespace pars {
namespace scan_detail {

constexpr unsigned kFull = 0xFFFFFFFFu;

// ---- fast-path automaton element -------------------------------------------
// State: bit0 e = "next byte is escaped", bit1 p = "inside a string".
// Element (a, b, q, d) maps (e, p) -> (a&e ^ b, p ^ q ^ d&e); bits a=0 b=1 q=2 d=3.
// Parity-only descriptors use a=1, b=0, d=0: p -> p ^ q.
constexpr std::uint32_t kIdent = 1u;

__device__ __forceinline__ std::uint32_t compose_fast(std::uint32_t X, std::uint32_t Y) {
	const std::uint32_t aX = X & 1u, bX = (X >> 1) & 1u, qX = (X >> 2) & 1u, dX = (X >> 3) & 1u;
	const std::uint32_t aY = Y & 1u, bY = (Y >> 1) & 1u, qY = (Y >> 2) & 1u, dY = (Y >> 3) & 1u;
	return (aX & aY) | (((bX & aY) ^ bY) << 1) | ((qX ^ qY ^ (bX & dY)) << 2)
		 | ((dX ^ (aX & dY)) << 3);
}

__device__ __forceinline__ std::uint32_t apply_fast(std::uint32_t X, std::uint32_t s) {
	const std::uint32_t e = s & 1u, p = (s >> 1) & 1u;
	const std::uint32_t a = X & 1u, b = (X >> 1) & 1u, q = (X >> 2) & 1u, d = (X >> 3) & 1u;
	return ((a & e) ^ b) | ((p ^ q ^ (d & e)) << 1);
}

// ---- R1: classify 32 bytes through the per-lane replicated table ----------------
// tbl_lane: shared-window byte address of column `lane` of a [256][32] u32 table.
// Each entry holds flag planes at bits 0 / 8 / 16 / 24; 8 consecutive lookups are
// summed with shifts (no carries), then a 4x4 byte transpose yields the planes.
__device__ __forceinline__ void classify32(const std::uint32_t (&r)[8], std::uint32_t tbl_lane,
										   std::uint32_t& P0, std::uint32_t& P1,
										   std::uint32_t& P2, std::uint32_t& P3) {
	std::uint32_t acc[4];
#pragma unroll
	for (int g = 0; g < 4; ++g) {
		std::uint32_t a = 0;
#pragma unroll
		for (int jj = 0; jj < 8; ++jj) {
			const int			j	= g * 8 + jj;
			const std::uint32_t w	= r[j >> 2];
			const int			k	= j & 3;
			std::uint32_t		off = (k == 0) ? (w << 7) : (w >> (8 * k - 7));
			off						= (off & 0x7F80u) + tbl_lane;
			std::uint32_t v;
			asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(off));
			a += v << jj;
		}
		acc[g] = a;
	}
	const std::uint32_t t0 = __byte_perm(acc[0], acc[1], 0x5140);
	const std::uint32_t t1 = __byte_perm(acc[0], acc[1], 0x7362);
	const std::uint32_t t2 = __byte_perm(acc[2], acc[3], 0x5140);
	const std::uint32_t t3 = __byte_perm(acc[2], acc[3], 0x7362);
	P0					   = __byte_perm(t0, t2, 0x5410);
	P1					   = __byte_perm(t0, t2, 0x7632);
	P2					   = __byte_perm(t1, t3, 0x5410);
	P3					   = __byte_perm(t1, t3, 0x7632);
}

// Exact SWAR byte-equality of 32 bytes against a replicated byte; 1 bit per byte.
__device__ __forceinline__ std::uint32_t eq_mask32(const std::uint32_t (&r)[8], std::uint32_t rep) {
	std::uint32_t m = 0;
#pragma unroll
	for (int i = 0; i < 8; ++i) {
		const std::uint32_t t = r[i] ^ rep;
		const std::uint32_t y = (t & 0x7F7F7F7Fu) + 0x7F7F7F7Fu;
		const std::uint32_t z = ~(y | t) & 0x80808080u;
		m |= ((z * 0x00204081u) >> 28) << (4 * i);
	}
	return m;
}

// Loads this thread's 32-byte word from a shared stage; the two 16-byte halves are
// read in swapped order on alternate quarter-warps so each LDS.128 phase hits all
// 32 banks.
__device__ __forceinline__ void load_word(const unsigned char* stage, int tid, std::uint32_t (&r)[8]) {
	const int	 sw = (tid >> 2) & 1;
	const uint4* p	= reinterpret_cast<const uint4*>(stage + 32 * tid);
	const uint4	 x	= p[sw];
	const uint4	 y	= p[sw ^ 1];
	const uint4	 h0 = sw ? y : x;
	const uint4	 h1 = sw ? x : y;
	r[0] = h0.x;
	r[1] = h0.y;
	r[2] = h0.z;
	r[3] = h0.w;
	r[4] = h1.x;
	r[5] = h1.y;
	r[6] = h1.z;
	r[7] = h1.w;
}

template<class T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
	for (int off = 16; off > 0; off >>= 1) {
		const T o = __shfl_xor_sync(kFull, v, off);
		v		  = o < v ? o : v;
	}
	return v;
}

template<class T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
	for (int off = 16; off > 0; off >>= 1) {
		const T o = __shfl_xor_sync(kFull, v, off);
		v		  = o > v ? o : v;
	}
	return v;
}

__device__ __forceinline__ void fence_acq_rel() {
	asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

}  // namespace scan_detail
}  // namespace pars
