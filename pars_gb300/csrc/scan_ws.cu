// scan_ws.cu — warp-specialised fused R1..R5 scan for plans whose lexical layer is
// empty, a quote-parity automaton or a doubled-delimiter automaton (the CSV shape).
//
// Each CTA runs 16 worker warps and one manager warp on a static tile schedule
// (CTA b owns 16 KiB tiles b, b+G, ...; cooperative launch keeps all CTAs
// resident).  Nothing waits on a CTA-wide barrier inside the tile loop: the warps
// hand work to each other through shared-memory mbarriers.
//
//   workers  A(k): wait for tile k's bytes (TMA ring), classify their 32-byte
//                  words, scan (in-string parity, counts under both parity
//                  hypotheses) across the warp, post the warp total, arrive TOT[k].
//            B(k): wait BASE[k], add the manager's cross-warp prefix, resolve the
//                  masks, write offsets / brackets / depth keys, arrive EMPTY[slot].
//            order: A(0), A(1), B(0), A(2), B(1), ... so the manager's look-back
//            for tile k overlaps the workers' classification of tile k+1.
//   manager  per tile: wait TOT[k], scan the 16 warp totals, publish the tile's AGG
//            look-back word, fold the predecessors' words, publish INCL, post the
//            tile base, arrive BASE[k]; refill ring slots as EMPTY completes.
//
// Look-back words and their fold are those of scan_fast.cu (fast_common.cuh).
// Reference semantics: include/pars/model/scan.hpp:33-72 and nest.hpp:55-76.
#include <cuda_runtime.h>

#include "fast_common.cuh"

namespace pars {

using namespace scan_detail;

namespace {

constexpr int kWorkers	 = 16;
constexpr int kWsThreads = (kWorkers + 1) * 32;
constexpr int kMgr		 = kWorkers;  // warp index of the manager

__device__ __forceinline__ void mbar_arrive(std::uint64_t* bar) {
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Bounded wait on the completion of phase `parity` of `bar`.
__device__ __forceinline__ bool mbar_wait(std::uint64_t* bar, std::uint32_t parity, DevResult* res) {
	std::uint32_t spins = 0;
	while (!mbar_try_wait(bar, parity)) {
		if (++spins > kSpinLimit) {
			record_error(res, kDevErrTimeout);
			return false;
		}
		if ((spins & 255u) == 0 && aborted(res))
			return false;
	}
	return true;
}

struct WsScratch {
	std::uint32_t wtot[2][kWorkers][4];	 // worker warp aggregates (workers -> manager)
	std::uint32_t wpre[2][kWorkers][4];	 // worker warp exclusive prefixes (manager -> workers)
	std::uint32_t state[2];				 // tile incoming state
	std::uint32_t base[2][3];			 // tile base counts
	std::uint32_t failed;
	std::uint32_t any_br;
	long long	  wext[4][kWorkers];
};

struct WsFront {
	std::uint32_t S, O, C, D;
	std::uint32_t ex0, dd;
	std::uint32_t ex[4];  // warp-exclusive scan value
	std::uint32_t vm;
};

struct SmemWs {
	static constexpr int kStage	   = 0;
	static constexpr int kBars	   = kStage + kRing * kTileBytes;	// full[3] empty[3] tot[2] base[2]
	static constexpr int kScratch  = kBars + 128;
	static constexpr int kHist	   = (kScratch + static_cast<int>(sizeof(WsScratch)) + 127) & ~127;
	static constexpr int kLowEnd   = kHist + 2 * kKeyWindow * 4;
	static constexpr int kTblBytes = 256 * 256;
	static constexpr int kBytes	   = kLowEnd + 65536 + kTblBytes;
};

struct OpSum3 {
	__device__ __forceinline__ void operator()(const std::uint32_t (&a)[4], std::uint32_t (&b)[4]) const {
		b[0] += a[0];
		b[2] += a[2];
		b[3] += a[3];
	}
};

// Warp-inclusive scan (lane order); N lanes of the value used.
template<class Op>
__device__ __forceinline__ void warp_scan(std::uint32_t (&x)[4], Op op, int lane, int n_active) {
#pragma unroll
	for (int off = 1; off < 32; off <<= 1) {
		if (off >= n_active)
			break;
		std::uint32_t y[4];
#pragma unroll
		for (int i = 0; i < 4; ++i) y[i] = __shfl_up_sync(kFull, x[i], off);
		if (lane >= off)
			op(y, x);
	}
}

}  // namespace

template<int PATH, bool BR>
__global__ void __launch_bounds__(kWsThreads, 1) k_scan_ws(const ScanArgs a) {
	extern __shared__ __align__(128) unsigned char smem[];
	unsigned char* ring		= smem + SmemWs::kStage;
	std::uint64_t* full_bar = reinterpret_cast<std::uint64_t*>(smem + SmemWs::kBars);
	std::uint64_t* empty_bar = full_bar + 3;
	std::uint64_t* tot_bar	 = full_bar + 6;
	std::uint64_t* base_bar	 = full_bar + 8;
	WsScratch&	   sc		 = *reinterpret_cast<WsScratch*>(smem + SmemWs::kScratch);
	unsigned int*  khist	 = reinterpret_cast<unsigned int*>(smem + SmemWs::kHist);
	const std::uint32_t win0	= smem_addr(smem);
	const std::uint32_t tbl_win = (win0 + SmemWs::kLowEnd + 0xFFFFu) & ~0xFFFFu;
	std::uint32_t*		tbl		= reinterpret_cast<std::uint32_t*>(smem + (tbl_win - win0));

	const int			tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const DevPlan*		P	= a.plan;
	DevResult*			res = a.res;
	uint4*				d_agg  = static_cast<uint4*>(a.tiles);
	uint4*				d_incl = d_agg + a.ntiles;
	const std::uint32_t G	   = gridDim.x;
	const std::uint32_t epoch  = a.epoch & 0x3FFFFFu;
	const std::uint32_t ntiles = static_cast<std::uint32_t>(a.ntiles);
	const unsigned long long doc_end = a.o + a.n;
	const std::uint32_t byte_base = a.carry_in ? static_cast<std::uint32_t>(a.carry_in->byte_base) : 0u;
	const std::uint32_t init_state = a.carry_in ? (a.carry_in->fstate & 3u) : 0u;
	const std::uint32_t base0[3] = {
		a.carry_in ? static_cast<std::uint32_t>(a.carry_in->ns) : 0u,
		a.carry_in ? static_cast<std::uint32_t>(a.carry_in->no) : 0u,
		a.carry_in ? static_cast<std::uint32_t>(a.carry_in->nc) : 0u};

	for (int i = tid; i < 256 * 32; i += kWsThreads) tbl[(i >> 5) * 64 + (i & 31)] = P->cls[i >> 5];
	if (BR)
		for (int i = tid; i < 2 * kKeyWindow; i += kWsThreads) khist[i] = 0;
	if (tid == 0) {
		for (int s = 0; s < 3; ++s) {
			mbar_init(&full_bar[s], 1);
			mbar_init(&empty_bar[s], kWorkers);
		}
		for (int p = 0; p < 2; ++p) {
			mbar_init(&tot_bar[p], kWorkers);
			mbar_init(&base_bar[p], 1);
		}
		fence_barrier_init();
		sc.failed = 0;
		if (tbl_win + SmemWs::kTblBytes > win0 + SmemWs::kBytes) {
			record_error(res, kDevErrTimeout);
			sc.failed = 1;
		}
	}
	__syncthreads();
	if (sc.failed)
		return;

	const std::uint32_t my_first = blockIdx.x;
	const std::uint32_t n_mine	 = my_first < ntiles ? (ntiles - 1 - my_first) / G + 1 : 0u;
	auto tile_of = [&](std::uint32_t k) { return my_first + k * G; };

	long long ext_min_bal = 0, ext_max_bal = 0;
	long long ext_min_key = 0x7FFFFFFFFFFFFFFFll, ext_max_key = -0x7FFFFFFFFFFFFFFFll;
	bool	  any_keys = false;

	if (warp == kMgr) {
		// ================================================================ manager ====
		std::uint32_t issued = 0;
		auto issue = [&](std::uint32_t k) {	 // lane 0
			if (k >= n_mine)
				return;
			issued					 = k + 1;
			const int				 s = static_cast<int>(k % 3);
			const unsigned long long off = static_cast<unsigned long long>(tile_of(k)) * kTileBytes;
			unsigned long long		 bytes = a.copy_end - off;
			if (bytes > kTileBytes)
				bytes = kTileBytes;
			mbar_arrive_expect_tx(&full_bar[s], static_cast<std::uint32_t>(bytes));
			bulk_g2s(ring + s * kTileBytes, a.base + off, static_cast<std::uint32_t>(bytes), &full_bar[s]);
		};
		if (lane == 0)
			for (std::uint32_t k = 0; k < 3; ++k) issue(k);
		bool failed = false;
		for (std::uint32_t k = 0; k < n_mine; ++k) {
			const std::uint32_t t	= tile_of(k);
			const int			buf = static_cast<int>(k & 1);
			if (!failed && !mbar_wait(&tot_bar[buf], (k >> 1) & 1u, res))
				failed = true;
			std::uint32_t s_t = init_state, base[3] = {base0[0], base0[1], base0[2]};
			uint4		  agg = make_uint4(0, 0, 0, 0);
			std::uint32_t tile_elem = kIdent;
			if (!failed) {
				// cross-warp exclusive scan of the 16 worker aggregates
				std::uint32_t w[4] = {0, 0, 0, 0};
				if (lane < kWorkers)
#pragma unroll
					for (int i = 0; i < 4; ++i) w[i] = sc.wtot[buf][lane][i];
				if (PATH == kPathNone)
					warp_scan(w, OpSum3(), lane, kWorkers);
				else
					warp_scan(w, OpParity(), lane, kWorkers);
				std::uint32_t we[4];
#pragma unroll
				for (int i = 0; i < 4; ++i) we[i] = __shfl_up_sync(kFull, w[i], 1);
				if (lane == 0)
#pragma unroll
					for (int i = 0; i < 4; ++i) we[i] = 0;
				if (lane < kWorkers)
#pragma unroll
					for (int i = 0; i < 4; ++i) sc.wpre[buf][lane][i] = we[i];
				std::uint32_t tot[4];
#pragma unroll
				for (int i = 0; i < 4; ++i) tot[i] = __shfl_sync(kFull, w[i], kWorkers - 1);
				if (PATH == kPathNone) {
					agg = make_uint4(tot[0], tot[2], tot[3], 0u);
				} else {
					tile_elem = 1u | (tot[1] << 2);
					agg		  = make_uint4(tot[0], tot[2], tot[3], tile_elem & 0xFu);
				}
				if (t == 0) {
					if (lane == 0) {
						std::uint32_t cs, co, cc;
						agg_counts<PATH>(agg, init_state, cs, co, cc);
						const std::uint32_t after = PATH == kPathNone ? 0u : apply_fast(tile_elem, init_state);
						st128_relaxed(&d_incl[0], make_uint4(base0[0] + cs, base0[1] + co, base0[2] + cc,
															 kDIncl | (epoch << 8) | after));
					}
				} else {
					if (lane == 0) {
						uint4 d = agg;
						d.w |= kDAgg | (epoch << 8);
						st128_relaxed(&d_agg[t], d);
					}
					// look-back: lane l holds distances j = l*kLB + i (j = 0 is tile t-1)
					const std::uint32_t W = t < G ? t : G;
					uint4				lbv[kLB];
#pragma unroll
					for (int i = 0; i < kLB; ++i) {
						const std::uint32_t j = static_cast<std::uint32_t>(lane) * kLB + i;
						lbv[i]				  = make_uint4(0, 0, 0, 0);
						if (j + 1 < W)
							lbv[i] = ld128_relaxed(&d_agg[t - 1 - j]);
						else if (j + 1 == W)
							lbv[i] = ld128_relaxed(&d_incl[t - W]);
					}
					bool bad = false;
#pragma unroll
					for (int i = 0; i < kLB; ++i) {
						const std::uint32_t j = static_cast<std::uint32_t>(lane) * kLB + i;
						if (j < W && !bad) {
							const bool			incl_slot = (j + 1 == W);
							const uint4*		src = incl_slot ? &d_incl[t - W] : &d_agg[t - 1 - j];
							const std::uint32_t want = incl_slot ? 2u : 1u;
							std::uint32_t		spins = 0;
							while (!((lbv[i].w >> 30) == want && ((lbv[i].w >> 8) & 0x3FFFFFu) == epoch)) {
								if (++spins > kSpinLimit) {
									record_error(res, kDevErrTimeout);
									bad = true;
									break;
								}
								if ((spins & 63u) == 0 && aborted(res)) {
									bad = true;
									break;
								}
								__nanosleep(32);
								lbv[i] = ld128_relaxed(src);
							}
						}
					}
					if (__any_sync(kFull, bad)) {
						failed = true;
					} else {
						std::uint32_t s_incl = 0, c_incl[3] = {0, 0, 0};
#pragma unroll
						for (int i = 0; i < kLB; ++i)
							if (static_cast<std::uint32_t>(lane) * kLB + i + 1 == W) {
								s_incl	  = lbv[i].w & 3u;
								c_incl[0] = lbv[i].x;
								c_incl[1] = lbv[i].y;
								c_incl[2] = lbv[i].z;
							}
						const int src_lane = static_cast<int>((W - 1) / kLB);
						s_incl			   = __shfl_sync(kFull, s_incl, src_lane);
						c_incl[0]		   = __shfl_sync(kFull, c_incl[0], src_lane);
						c_incl[1]		   = __shfl_sync(kFull, c_incl[1], src_lane);
						c_incl[2]		   = __shfl_sync(kFull, c_incl[2], src_lane);
						std::uint32_t E	   = kIdent;
#pragma unroll
						for (int i = kLB - 1; i >= 0; --i)
							if (static_cast<std::uint32_t>(lane) * kLB + i + 1 < W)
								E = compose_fast(E, lbv[i].w & 0xFu);
						std::uint32_t x = E;
#pragma unroll
						for (int off = 1; off < 32; off <<= 1) {
							const std::uint32_t o = __shfl_down_sync(kFull, x, off);
							if (lane + off < 32)
								x = compose_fast(o, x);
						}
						std::uint32_t ex = __shfl_down_sync(kFull, x, 1);
						if (lane == 31)
							ex = kIdent;
						std::uint32_t st = PATH == kPathNone ? 0u : apply_fast(ex, s_incl);
						std::uint32_t cs = 0, co = 0, cc = 0;
#pragma unroll
						for (int i = kLB - 1; i >= 0; --i)
							if (static_cast<std::uint32_t>(lane) * kLB + i + 1 < W) {
								std::uint32_t a0, a1, a2;
								agg_counts<PATH>(lbv[i], st, a0, a1, a2);
								cs += a0;
								co += a1;
								cc += a2;
								if (PATH != kPathNone)
									st = apply_fast(lbv[i].w & 0xFu, st);
							}
#pragma unroll
						for (int off = 16; off > 0; off >>= 1) {
							cs += __shfl_xor_sync(kFull, cs, off);
							if (BR) {
								co += __shfl_xor_sync(kFull, co, off);
								cc += __shfl_xor_sync(kFull, cc, off);
							}
						}
						s_t		= __shfl_sync(kFull, st, 0);
						base[0] = c_incl[0] + cs;
						base[1] = c_incl[1] + co;
						base[2] = c_incl[2] + cc;
						if (lane == 0) {
							std::uint32_t c0, c1, c2;
							agg_counts<PATH>(agg, s_t, c0, c1, c2);
							const std::uint32_t after = PATH == kPathNone ? 0u : apply_fast(tile_elem, s_t);
							st128_relaxed(&d_incl[t], make_uint4(base[0] + c0, base[1] + c1, base[2] + c2,
																 kDIncl | (epoch << 8) | after));
						}
					}
				}
			}
			if (lane == 0) {
				if (failed)
					sc.failed = 1;
				sc.state[buf]	= s_t;
				sc.base[buf][0] = base[0];
				sc.base[buf][1] = base[1];
				sc.base[buf][2] = base[2];
				if (!failed && t == ntiles - 1) {
					std::uint32_t c0, c1, c2;
					agg_counts<PATH>(agg, s_t, c0, c1, c2);
					const unsigned long long ns = static_cast<unsigned long long>(base[0]) + c0;
					const unsigned long long no = static_cast<unsigned long long>(base[1]) + c1;
					const unsigned long long nc = static_cast<unsigned long long>(base[2]) + c2;
					res->n_struct	= ns;
					res->n_open		= no;
					res->n_close	= nc;
					res->n_brackets = no + nc;
					res->path		= PATH;
					if (a.carry_out) {
						a.carry_out->ns		   = ns;
						a.carry_out->no		   = no;
						a.carry_out->nc		   = nc;
						a.carry_out->byte_base = byte_base + a.n;
					}
				}
			}
			__syncwarp();
			if (lane == 0)
				mbar_arrive(&base_bar[buf]);
			// ring refill: tile k-1's slot takes tile k+2 once its workers are done
			if (lane == 0 && !failed && k >= 1 && k + 2 < n_mine) {
				if (mbar_wait(&empty_bar[(k - 1) % 3], ((k - 1) / 3) & 1u, res))
					issue(k + 2);
				else
					failed = true;
			}
			failed = __shfl_sync(kFull, failed ? 1u : 0u, 0) != 0;
		}
		// drain: every issued copy must land before the CTA exits
		if (lane == 0)
			for (std::uint32_t k = (issued > 3 ? issued - 3 : 0); k < issued; ++k)
				mbar_wait(&full_bar[k % 3], (k / 3) & 1u, res);
	} else {
		// ================================================================ workers ====
		const std::uint32_t wtid	 = static_cast<std::uint32_t>(tid);	 // 0..511
		const std::uint32_t tbl_lane = tbl_win + 4u * lane;
		const std::uint32_t sw		 = (wtid >> 2) & 1u;
		const std::uint32_t selA	 = sw ? 0x1054u : 0x5410u;
		const std::uint32_t selB	 = sw ? 0x3276u : 0x7632u;
		const std::uint8_t	delim	 = P->delim;
		const bool			want_pairs = (a.flags & 1u) != 0;
		const bool			want_chars = (a.flags & 4u) != 0;
		const bool			want_mask  = (a.flags & 8u) != 0 && a.mask;
		const std::uint32_t cap_s = a.cap_s > 0xFFFFFFFFull ? 0xFFFFFFFFu : static_cast<std::uint32_t>(a.cap_s);
		const std::uint32_t cap_b = a.cap_b > 0xFFFFFFFFull ? 0xFFFFFFFFu : static_cast<std::uint32_t>(a.cap_b);

		auto phase_a = [&](std::uint32_t k, WsFront& F) -> bool {
			const std::uint32_t t	= tile_of(k);
			const int			s	= static_cast<int>(k % 3);
			const int			buf = static_cast<int>(k & 1);
			if (!mbar_wait(&full_bar[s], (k / 3) & 1u, res)) {
				sc.failed = 1;
				return false;
			}
			const unsigned char*	 stage = ring + s * kTileBytes;
			const unsigned long long q0	   = static_cast<unsigned long long>(t) * kTileBytes + 32u * wtid;
			const bool interior = static_cast<unsigned long long>(t) * kTileBytes >= a.o
							   && static_cast<unsigned long long>(t + 1) * kTileBytes <= doc_end;
			std::uint32_t vm = 0xFFFFFFFFu;
			int			  lo = 0, hi = 32;
			if (!interior) {
				if (q0 < a.o)
					lo = (a.o - q0) > 32 ? 32 : static_cast<int>(a.o - q0);
				if (doc_end < q0 + 32)
					hi = doc_end <= q0 ? 0 : static_cast<int>(doc_end - q0);
				if (hi < lo)
					hi = lo;
				vm = bit_range(lo, hi);
			}
			F.vm = vm;
			std::uint32_t r[8];
			{
				const uint4* p = reinterpret_cast<const uint4*>(stage + 32 * wtid);
				const uint4	 x = p[sw];
				const uint4	 y = p[sw ^ 1u];
				r[0] = x.x;
				r[1] = x.y;
				r[2] = x.z;
				r[3] = x.w;
				r[4] = y.x;
				r[5] = y.y;
				r[6] = y.z;
				r[7] = y.w;
			}
			std::uint32_t S, O, C, D;
			classify_word(r, tbl_lane, selA, selB, S, O, C, D);
			if (!interior) {
				S &= vm;
				O &= vm;
				C &= vm;
				D &= vm;
			}
			F.S = S;
			F.O = O;
			F.C = C;
			F.D = D;
			std::uint32_t v[4];
			if (PATH == kPathNone) {
				F.ex0 = F.dd = 0;
				v[0] = __popc(S);
				v[1] = 0;
				v[2] = BR ? __popc(O) : 0u;
				v[3] = BR ? __popc(C) : 0u;
				warp_scan(v, OpSum3(), lane, 32);
			} else {
				const std::uint32_t ex0 = prefix_xor32(D) ^ D;
				std::uint32_t		dd	= 0;
				if (PATH == kPathDoubled) {
					std::uint32_t prev	= __shfl_up_sync(kFull, D >> 31, 1);
					const bool	  first = (q0 + lo == a.o);
					if (first) {
						prev = a.carry_in ? (a.carry_in->last_delim & 1u) : 0u;
					} else if (lane == 0 && vm != 0) {
						prev = (wtid > 0 ? stage[32 * wtid - 1] : a.base[q0 - 1]) == delim ? 1u : 0u;
					}
					dd = D & ((D << 1) | ((prev & 1u) << lo));
				}
				const std::uint32_t m0 = ex0 | dd, m1 = ~ex0 | dd;
				v[0] = __popc(S & ~m0) | (__popc(S & ~m1) << 16);
				v[1] = __popc(D) & 1u;
				v[2] = BR ? (__popc(O & ~m0) | (__popc(O & ~m1) << 16)) : 0u;
				v[3] = BR ? (__popc(C & ~m0) | (__popc(C & ~m1) << 16)) : 0u;
				F.ex0 = ex0;
				F.dd  = dd;
				warp_scan(v, OpParity(), lane, 32);
			}
			// v is now warp-inclusive; keep the warp-exclusive part
#pragma unroll
			for (int i = 0; i < 4; ++i) {
				const std::uint32_t e = __shfl_up_sync(kFull, v[i], 1);
				F.ex[i]				  = lane == 0 ? 0u : e;
			}
			if (lane == 31)
#pragma unroll
				for (int i = 0; i < 4; ++i) sc.wtot[buf][warp][i] = v[i];
			__syncwarp();
			if (lane == 0)
				mbar_arrive(&tot_bar[buf]);
			return true;
		};

		auto phase_b = [&](std::uint32_t k, const WsFront& F) -> bool {
			const std::uint32_t t	= tile_of(k);
			const int			s	= static_cast<int>(k % 3);
			const int			buf = static_cast<int>(k & 1);
			if (!mbar_wait(&base_bar[buf], (k >> 1) & 1u, res) || sc.failed) {
				sc.failed = 1;
				return false;
			}
			const unsigned char*	 stage = ring + s * kTileBytes;
			const unsigned long long q0	   = static_cast<unsigned long long>(t) * kTileBytes + 32u * wtid;
			const std::uint32_t		 s_t   = sc.state[buf];
			const std::uint32_t		 p_t   = (s_t >> 1) & 1u;
			// this word's prefix = manager's cross-warp prefix, then the warp prefix
			std::uint32_t pre[4];
#pragma unroll
			for (int i = 0; i < 4; ++i) pre[i] = sc.wpre[buf][warp][i];
			std::uint32_t ex[4] = {F.ex[0], F.ex[1], F.ex[2], F.ex[3]};
			std::uint32_t off[3];
			std::uint32_t p_w = 0;
			if (PATH == kPathNone) {
				OpSum3()(pre, ex);
				off[0] = ex[0];
				off[1] = ex[2];
				off[2] = ex[3];
			} else {
				OpParity()(pre, ex);
				p_w	   = p_t ^ ex[1];
				off[0] = half16(ex[0], p_t);
				off[1] = half16(ex[2], p_t);
				off[2] = half16(ex[3], p_t);
			}
			const std::uint32_t base[3] = {sc.base[buf][0], sc.base[buf][1], sc.base[buf][2]};
			const std::uint32_t vm		= F.vm;
			std::uint32_t		mask	= 0;
			if (PATH != kPathNone)
				mask = ((F.ex0 ^ (p_w ? 0xFFFFFFFFu : 0u)) | F.dd) & vm;
			// the worker holding the document's last byte records the end state
			if (vm != 0 && doc_end <= q0 + 32 && doc_end > q0) {
				const int			hi		  = static_cast<int>(doc_end - q0);
				const std::uint32_t elem	  = 1u | ((__popc(F.D) & 1u) << 2);
				const std::uint32_t endstate  = PATH == kPathNone ? 0u : apply_fast(elem, p_w << 1);
				const std::uint32_t last_flag = (F.D >> (hi - 1)) & 1u;
				const std::uint32_t unclosed  = PATH == kPathNone ? 0u : (((endstate >> 1) & 1u) | last_flag);
				res->unclosed				  = unclosed;
				if (a.carry_out) {
					a.carry_out->fstate		 = endstate;
					a.carry_out->last_delim	 = last_flag;
					a.carry_out->last_toggle = last_flag;
					a.carry_out->unclosed	 = unclosed;
				}
			}
			std::uint32_t		m	 = F.S & ~mask;
			std::uint32_t		si	 = base[0] + off[0];
			const std::uint32_t pos0 = byte_base + static_cast<std::uint32_t>(q0 - a.o);
			const unsigned char* wb	 = stage + 32 * wtid;
			if (!BR) {
				if (si + static_cast<std::uint32_t>(__popc(m)) <= cap_s && !want_chars && !want_pairs) {
					std::uint32_t* out = a.pos + si;
					while (m) {
						const int j = __ffs(m) - 1;
						m &= m - 1;
						*out++ = pos0 + j;
					}
				} else {
					while (m) {
						const int j = __ffs(m) - 1;
						m &= m - 1;
						if (si < cap_s) {
							a.pos[si] = pos0 + j;
							if (want_chars)
								a.chars[si] = wb[j];
							if (want_pairs)
								a.pair[si] = -1;
						}
						++si;
					}
				}
			} else {
				const std::uint32_t selo = F.O & ~mask;
				const std::uint32_t selc = F.C & ~mask;
				const std::uint32_t no0	 = base[1] + off[1];
				const std::uint32_t nc0	 = base[2] + off[2];
				std::uint32_t		bi	 = no0 + nc0;
				long long			dep	 = static_cast<long long>(no0) - static_cast<long long>(nc0);
				const std::uint32_t bm	 = selo | selc;
				while (m) {
					const int j = __ffs(m) - 1;
					m &= m - 1;
					const std::uint32_t pos = pos0 + j;
					if (si < cap_s) {
						a.pos[si] = pos;
						if (want_chars)
							a.chars[si] = wb[j];
						if (want_pairs)
							a.pair[si] = -1;
					}
					if ((bm >> j) & 1u) {
						const bool		op	= (selo >> j) & 1u;
						const long long key = op ? dep : dep - 1;
						dep += op ? 1 : -1;
						if (bi < cap_b) {
							a.bpos[bi]	= pos;
							a.bchar[bi] = wb[j];
							a.bsi[bi]	= si;
							a.depth[bi] = static_cast<std::int32_t>(key);
						}
						++bi;
						ext_min_bal = dep < ext_min_bal ? dep : ext_min_bal;
						ext_max_bal = dep > ext_max_bal ? dep : ext_max_bal;
						ext_min_key = key < ext_min_key ? key : ext_min_key;
						ext_max_key = key > ext_max_key ? key : ext_max_key;
						any_keys	= true;
						if (key >= -kKeyWindow && key < kKeyWindow)
							atomicAdd(&khist[key + kKeyWindow], 1u);
						else
							atomicOr(&res->keys_oob, 1u);
					}
					++si;
				}
			}
			if (want_mask && vm != 0)
				a.mask[(byte_base + static_cast<std::uint32_t>(q0 - a.o)) >> 5] = mask;
			__syncwarp();
			if (lane == 0)
				mbar_arrive(&empty_bar[s]);
			return true;
		};

		WsFront f0, f1;
		bool	ok = n_mine > 0 ? phase_a(0, f0) : true;
		for (std::uint32_t k = 0; ok && k < n_mine; k += 2) {
			if (k + 1 < n_mine)
				ok = phase_a(k + 1, f1);
			if (!ok || !phase_b(k, f0))
				break;
			if (k + 1 >= n_mine)
				break;
			if (k + 2 < n_mine)
				ok = phase_a(k + 2, f0);
			if (!ok || !phase_b(k + 1, f1))
				break;
		}
	}
	__syncthreads();

	// ---- CTA exit: depth extrema and key histogram (workers) -------------------------
	if (BR) {
		if (tid == 0)
			sc.any_br = 0;
		__syncthreads();
		if (warp < kWorkers) {
			const long long v0 = warp_min(ext_min_bal), v1 = warp_max(ext_max_bal);
			const long long v2 = warp_min(ext_min_key), v3 = warp_max(ext_max_key);
			const bool		anyk = __any_sync(kFull, any_keys);
			if (lane == 0) {
				sc.wext[0][warp] = v0;
				sc.wext[1][warp] = v1;
				sc.wext[2][warp] = v2;
				sc.wext[3][warp] = v3;
				if (anyk)
					sc.any_br = 1;
			}
		}
		__syncthreads();
		if (tid == 0 && sc.any_br) {
			long long mn = 0, mx = 0, kn = 0x7FFFFFFFFFFFFFFFll, kx = -0x7FFFFFFFFFFFFFFFll;
			for (int w = 0; w < kWorkers; ++w) {
				mn = sc.wext[0][w] < mn ? sc.wext[0][w] : mn;
				mx = sc.wext[1][w] > mx ? sc.wext[1][w] : mx;
				kn = sc.wext[2][w] < kn ? sc.wext[2][w] : kn;
				kx = sc.wext[3][w] > kx ? sc.wext[3][w] : kx;
			}
			atomicMax(&res->min_bal, enc_min(mn));
			atomicMax(&res->max_bal, enc_max(mx));
			atomicMax(&res->min_key, enc_min(kn));
			atomicMax(&res->max_key, enc_max(kx));
		}
		if (sc.any_br)
			for (int i = tid; i < 2 * kKeyWindow; i += kWsThreads)
				if (khist[i])
					atomicAdd(&a.key_hist[i], khist[i]);
	}
}

#define PARS_INST(P, B) template __global__ void k_scan_ws<P, B>(const ScanArgs);
PARS_INST(kPathNone, false)
PARS_INST(kPathNone, true)
PARS_INST(kPathParity, false)
PARS_INST(kPathParity, true)
PARS_INST(kPathDoubled, false)
PARS_INST(kPathDoubled, true)
#undef PARS_INST

int scan_ws_threads() {
	return kWsThreads;
}

int scan_ws_smem_bytes() {
	return SmemWs::kBytes;
}

const void* scan_ws_kernel(int path, bool brackets) {
	switch (path * 2 + (brackets ? 1 : 0)) {
		case 0: return reinterpret_cast<const void*>(&k_scan_ws<kPathNone, false>);
		case 1: return reinterpret_cast<const void*>(&k_scan_ws<kPathNone, true>);
		case 2: return reinterpret_cast<const void*>(&k_scan_ws<kPathParity, false>);
		case 3: return reinterpret_cast<const void*>(&k_scan_ws<kPathParity, true>);
		case 4: return reinterpret_cast<const void*>(&k_scan_ws<kPathDoubled, false>);
		case 5: return reinterpret_cast<const void*>(&k_scan_ws<kPathDoubled, true>);
		default: return nullptr;
	}
}

}  // namespace pars
