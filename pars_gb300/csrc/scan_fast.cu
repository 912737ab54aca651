// scan_fast.cu — fused R1..R5 single-pass scan for plans with at most one lexical
// descriptor of a recognised shape (none / quote parity / doubled delimiter /
// prefix escape), i.e. the JSON and CSV grammars and their relatives.
//
// Schedule.  A cooperative (all CTAs co-resident) persistent grid of G CTAs walks
// the input in 16 KiB tiles with a static schedule: CTA b owns tiles b, b+G, ...
// Each CTA keeps three tiles in its shared-memory ring (1-D TMA bulk copies
// completing on mbarriers), and software-pipelines two of them:
//
//     issue look-back loads for tile k        (128-bit, relaxed)
//     phase A(k+1): classify, local scans, publish AGG(k+1)
//     finish look-back of tile k, publish INCL(k)
//     phase B(k): resolve masks, write offsets / brackets / depth keys
//
// so the L2 round trip of the look-back overlaps the classification of the next
// tile, and every predecessor a tile waits for has already published.
//
// Look-back descriptor (one 128-bit word per tile, single-copy atomic):
//   AGG : per-class counts of the tile under both in-string hypotheses (u16
//         halves), the tile's automaton element, and (escape path) the class of
//         the tile's first non-backslash byte;
//   INCL: the state after the tile and cumulative counts (u32 each);
//   w[31:30] flag, w[29:8] epoch of the launch, w[7:0] element / state bits.
//
// Reference semantics: include/pars/model/scan.hpp:33-72 and nest.hpp:55-76
// (see scan.cu for the generic descriptor kernel that runs every other plan).
#include <cuda_runtime.h>

#include "scan_common.cuh"

namespace pars {

using namespace scan_detail;

namespace {

constexpr std::uint32_t kDAgg  = 1u << 30;
constexpr std::uint32_t kDIncl = 2u << 30;
constexpr int			kWarps = kScanThreads / 32;
constexpr int			kRing  = 3;

__device__ __forceinline__ std::uint32_t half16(std::uint32_t x, std::uint32_t h) {
	return h ? (x >> 16) : (x & 0xFFFFu);
}

// Counts of a tile (AGG payload) when it is entered in state s = (e, p).
template<int PATH>
__device__ __forceinline__ void agg_counts(const uint4& v, std::uint32_t s, std::uint32_t& cs,
										   std::uint32_t& co, std::uint32_t& cc) {
	if (PATH == kPathNone) {
		cs = v.x;
		co = v.y;
		cc = v.z;
		return;
	}
	const std::uint32_t e = s & 1u, p = (s >> 1) & 1u;
	const std::uint32_t d	 = (v.w >> 3) & 1u;
	const std::uint32_t fcl	 = (v.w >> 4) & 7u;
	const std::uint32_t h	 = p ^ (e & d);
	const std::uint32_t lo	 = p ? 0u : 1u;
	cs = half16(v.x, h) + ((fcl & 1u) ? lo : 0u);
	co = half16(v.y, h) + ((fcl & 2u) ? lo : 0u);
	cc = half16(v.z, h) + ((fcl & 4u) ? lo : 0u);
}

struct FastScratch {
	std::uint32_t wpart[2][kWarps + 1][4];	 // block-scan partials (+ total), per tile in flight
	std::uint32_t tile_elem[2];
	std::uint32_t tile_cnt[2][3];
	std::uint32_t fword[2];
	std::uint32_t fcls[2];
	std::uint32_t dt[2];
	// look-back fold
	std::uint32_t fold_J;
	std::uint32_t incl_state;
	std::uint32_t incl_cnt[3];
	std::uint32_t warp_elem[kWarps];
	std::uint32_t warp_sum[kWarps][3];
	std::uint32_t s_enter[kWarps];
	std::uint32_t in_state;
	std::uint32_t base[3];
	std::uint32_t failed;
	std::uint32_t any_br;
	long long	  wext[4][kWarps];
};

// Per-thread state of one tile between phase A and phase B.
struct Front {
	std::uint32_t S, O, C, D;
	std::uint32_t ex0;	 // exclusive in-string parity of the word (escape: with e = 0)
	std::uint32_t aux;	 // doubled: D & previous-byte-delim; escape: escaped bytes with e = 0
	std::uint32_t fbit;	 // escape: lowest valid non-backslash byte
	std::uint32_t pre;	 // exclusive element of the word within the tile
	std::uint32_t elem;	 // the word's own element
	std::uint32_t off[3];
	int			  lo, hi;
};

struct SmemFast {
	static constexpr int kTbl	  = 0;
	static constexpr int kStage	  = kTbl + 256 * 32 * 4;
	static constexpr int kBars	  = kStage + kRing * kTileBytes;
	static constexpr int kScratch = kBars + 64;
	static constexpr int kHist	  = (kScratch + static_cast<int>(sizeof(FastScratch)) + 127) & ~127;
	static constexpr int kBytes	  = kHist + 2 * kKeyWindow * 4;
};

// ---- block-wide helpers ----------------------------------------------------------
// Exclusive scan of up to 4 u32 lanes with an associative op; `total` gets the
// block aggregate.  Two __syncthreads.
template<int N, class Op>
__device__ __forceinline__ void block_scan(std::uint32_t (&v)[4], std::uint32_t (&excl)[4],
										   std::uint32_t (&total)[4], const std::uint32_t (&ident)[4],
										   Op op, std::uint32_t (*wpart)[4]) {
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	std::uint32_t x[4];
#pragma unroll
	for (int i = 0; i < 4; ++i) x[i] = v[i];
#pragma unroll
	for (int off = 1; off < 32; off <<= 1) {
		std::uint32_t y[4];
#pragma unroll
		for (int i = 0; i < N; ++i) y[i] = __shfl_up_sync(kFull, x[i], off);
		if (lane >= off)
			op(y, x);  // x = y (earlier) then x
	}
	std::uint32_t ex[4];
#pragma unroll
	for (int i = 0; i < N; ++i) ex[i] = __shfl_up_sync(kFull, x[i], 1);
	if (lane == 0)
#pragma unroll
		for (int i = 0; i < N; ++i) ex[i] = ident[i];
	if (lane == 31)
#pragma unroll
		for (int i = 0; i < N; ++i) wpart[warp][i] = x[i];
	__syncthreads();
	if (warp == 0) {
		std::uint32_t w[4];
#pragma unroll
		for (int i = 0; i < N; ++i) w[i] = lane < kWarps ? wpart[lane][i] : ident[i];
#pragma unroll
		for (int off = 1; off < kWarps; off <<= 1) {
			std::uint32_t y[4];
#pragma unroll
			for (int i = 0; i < N; ++i) y[i] = __shfl_up_sync(kFull, w[i], off);
			if (lane >= off)
				op(y, w);
		}
		std::uint32_t we[4];
#pragma unroll
		for (int i = 0; i < N; ++i) we[i] = __shfl_up_sync(kFull, w[i], 1);
		if (lane == 0)
#pragma unroll
			for (int i = 0; i < N; ++i) we[i] = ident[i];
		__syncwarp();
		if (lane < kWarps)
#pragma unroll
			for (int i = 0; i < N; ++i) wpart[lane][i] = we[i];
		if (lane == kWarps - 1)
#pragma unroll
			for (int i = 0; i < N; ++i) wpart[kWarps][i] = w[i];
	}
	__syncthreads();
	std::uint32_t wp[4];
#pragma unroll
	for (int i = 0; i < N; ++i) {
		wp[i]	 = wpart[warp][i];
		total[i] = wpart[kWarps][i];
	}
	// excl = wp (earlier warps) then ex (earlier lanes)
	op(wp, ex);
#pragma unroll
	for (int i = 0; i < N; ++i) excl[i] = ex[i];
}

struct OpSum3 {
	__device__ __forceinline__ void operator()(const std::uint32_t (&a)[4], std::uint32_t (&b)[4]) const {
		b[0] += a[0];
		b[1] += a[1];
		b[2] += a[2];
	}
};

// (parity bit, packed counts under hypotheses 0/1): a then b.
struct OpParity {
	__device__ __forceinline__ void operator()(const std::uint32_t (&a)[4], std::uint32_t (&b)[4]) const {
		const std::uint32_t sw = a[3] ? 0x1032u : 0x3210u;
		b[0] = a[0] + __byte_perm(b[0], 0, sw);
		b[1] = a[1] + __byte_perm(b[1], 0, sw);
		b[2] = a[2] + __byte_perm(b[2], 0, sw);
		b[3] ^= a[3];
	}
};

struct OpElem {
	__device__ __forceinline__ void operator()(const std::uint32_t (&a)[4], std::uint32_t (&b)[4]) const {
		b[0] = compose_fast(a[0], b[0]);
	}
};

}  // namespace

// ============================================================================
template<int PATH, bool BR>
__global__ void __launch_bounds__(kScanThreads, 1) k_scan_fast(const ScanArgs a) {
	extern __shared__ __align__(128) unsigned char smem[];
	std::uint32_t* tbl	  = reinterpret_cast<std::uint32_t*>(smem + SmemFast::kTbl);
	unsigned char* ring	  = smem + SmemFast::kStage;
	std::uint64_t* bars	  = reinterpret_cast<std::uint64_t*>(smem + SmemFast::kBars);
	FastScratch&   sc	  = *reinterpret_cast<FastScratch*>(smem + SmemFast::kScratch);
	unsigned int*  khist  = reinterpret_cast<unsigned int*>(smem + SmemFast::kHist);

	const int			tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const DevPlan*		P	= a.plan;
	DevResult*			res = a.res;
	uint4*				desc = static_cast<uint4*>(a.tiles);
	const unsigned long long G	   = gridDim.x;
	const std::uint32_t epoch	   = a.epoch & 0x3FFFFFu;
	const unsigned long long doc_end   = a.o + a.n;
	const unsigned long long byte_base = a.carry_in ? a.carry_in->byte_base : 0ull;
	const std::uint32_t init_state = a.carry_in ? (a.carry_in->fstate & 3u) : 0u;
	const std::uint32_t base0[3] = {
		a.carry_in ? static_cast<std::uint32_t>(a.carry_in->ns) : 0u,
		a.carry_in ? static_cast<std::uint32_t>(a.carry_in->no) : 0u,
		a.carry_in ? static_cast<std::uint32_t>(a.carry_in->nc) : 0u};
	const std::uint32_t escape_rep = P->escape_rep;
	const std::uint8_t	delim	   = P->delim;
	const bool			want_pairs = (a.flags & 1u) != 0;
	const bool			want_chars = (a.flags & 4u) != 0;
	const bool			want_mask  = (a.flags & 8u) != 0 && a.mask;

	for (int i = tid; i < 256 * 32; i += kScanThreads) tbl[i] = P->cls[i >> 5];
	if (BR)
		for (int i = tid; i < 2 * kKeyWindow; i += kScanThreads) khist[i] = 0;
	if (tid == 0) {
		for (int s = 0; s < kRing; ++s) mbar_init(&bars[s], 1);
		fence_barrier_init();
		sc.failed = 0;
	}
	__syncthreads();

	// my tiles: t_k = blockIdx.x + k * G
	const unsigned long long my_first = blockIdx.x;
	const unsigned long long n_mine =
		my_first < a.ntiles ? (a.ntiles - 1 - my_first) / G + 1 : 0ull;
	auto tile_of = [&](unsigned long long k) { return my_first + k * G; };
	unsigned long long issued = 0, waited = 0;	// tid 0: copies started / consumed
	auto issue = [&](unsigned long long k) {  // tid 0: start the copy of my k-th tile
		if (k >= n_mine)
			return;
		issued = k + 1;
		const int				 s	   = static_cast<int>(k % kRing);
		const unsigned long long off   = tile_of(k) * kTileBytes;
		unsigned long long		 bytes = a.copy_end - off;
		if (bytes > kTileBytes)
			bytes = kTileBytes;
		mbar_arrive_expect_tx(&bars[s], static_cast<std::uint32_t>(bytes));
		bulk_g2s(ring + s * kTileBytes, a.base + off, static_cast<std::uint32_t>(bytes), &bars[s]);
	};
	if (tid == 0)
		for (int k = 0; k < kRing; ++k) issue(k);

	const std::uint32_t tbl_lane = smem_addr(tbl) + 4u * lane;
	std::uint32_t		phase_bits = 0;
	long long			ext_min_bal = 0, ext_max_bal = 0;
	long long			ext_min_key = 0x7FFFFFFFFFFFFFFFll, ext_max_key = -0x7FFFFFFFFFFFFFFFll;
	bool				any_keys = false;

	// ---------------------------------------------------------------- phase A ----
	auto phase_a = [&](unsigned long long k, Front& F) {
		const unsigned long long t	 = tile_of(k);
		const int				 s	 = static_cast<int>(k % kRing);
		const int				 buf = static_cast<int>(k & 1);
		{
			std::uint32_t spins = 0;
			while (!mbar_try_wait(&bars[s], (phase_bits >> s) & 1u)) {
				if (++spins > kSpinLimit) {
					record_error(res, kDevErrTimeout);
					sc.failed = 1;
					break;
				}
			}
			phase_bits ^= 1u << s;
			waited = k + 1;
		}
		const unsigned char*	 stage = ring + s * kTileBytes;
		const unsigned long long q0	   = t * kTileBytes + 32ull * tid;
		int lo = 0, hi = 32;
		if (q0 < a.o)
			lo = (a.o - q0) > 32 ? 32 : static_cast<int>(a.o - q0);
		if (doc_end < q0 + 32)
			hi = doc_end <= q0 ? 0 : static_cast<int>(doc_end - q0);
		if (hi < lo)
			hi = lo;
		F.lo					= lo;
		F.hi					= hi;
		const std::uint32_t vm = bit_range(lo, hi);
		std::uint32_t		r[8];
		load_word(stage, tid, r);
		std::uint32_t S, O, C, D;
		classify32(r, tbl_lane, S, O, C, D);
		S &= vm;
		O &= vm;
		C &= vm;
		D &= vm;
		F.S = S;
		F.O = O;
		F.C = C;
		F.D = D;
		F.aux = 0;
		F.fbit = 0;
		F.ex0 = 0;
		std::uint32_t v[4], ex[4], tot[4];
		if (PATH == kPathNone) {
			v[0] = __popc(S);
			v[1] = __popc(O);
			v[2] = __popc(C);
			v[3] = 0;
			const std::uint32_t id[4] = {0, 0, 0, 0};
			block_scan<3>(v, ex, tot, id, OpSum3(), sc.wpart[buf]);
			F.pre  = kIdent;
			F.elem = kIdent;
		} else if (PATH == kPathParity || PATH == kPathDoubled) {
			const std::uint32_t ex0 = prefix_xor32(D) ^ D;
			std::uint32_t		dd	= 0;
			if (PATH == kPathDoubled) {
				std::uint32_t prev	= __shfl_up_sync(kFull, D >> 31, 1);
				const bool	  first = (q0 + lo == a.o);
				if (first) {
					prev = a.carry_in ? (a.carry_in->last_delim & 1u) : 0u;
				} else if (lane == 0 && vm != 0) {
					prev = (tid > 0 ? stage[32 * tid - 1] : a.base[q0 - 1]) == delim ? 1u : 0u;
				}
				dd = D & ((D << 1) | ((prev & 1u) << lo));
			}
			const std::uint32_t m0 = ex0 | dd, m1 = ~ex0 | dd;
			v[0] = __popc(S & ~m0) | (__popc(S & ~m1) << 16);
			if (BR) {
				v[1] = __popc(O & ~m0) | (__popc(O & ~m1) << 16);
				v[2] = __popc(C & ~m0) | (__popc(C & ~m1) << 16);
			} else {
				v[1] = v[2] = 0;
			}
			v[3] = __popc(D) & 1u;
			const std::uint32_t id[4] = {0, 0, 0, 0};
			block_scan<4>(v, ex, tot, id, OpParity(), sc.wpart[buf]);
			F.ex0  = ex0;
			F.aux  = dd;
			F.pre  = 1u | (ex[3] << 2);
			F.elem = 1u | ((__popc(D) & 1u) << 2);
			tot[3] = 1u | (tot[3] << 2);  // tile element
		} else {  // kPathEscape
			const std::uint32_t B	 = eq_mask32(r, escape_rep) & vm;
			const std::uint32_t runs = B & ~(B << 1);
			const std::uint32_t ee	 = (B + (runs & 0x55555555u)) & ~B;
			const std::uint32_t eo	 = (B + (runs & 0xAAAAAAAAu)) & ~B;
			const std::uint32_t esc0 = (ee & 0xAAAAAAAAu) | (eo & 0x55555555u);
			const std::uint32_t nbv	 = ~B & vm;
			const std::uint32_t fbit = nbv & (0u - nbv);
			const std::uint32_t T0	 = D & ~esc0;
			const std::uint32_t ex0	 = prefix_xor32(T0) ^ T0;
			std::uint32_t		elem = kIdent;
			if (vm != 0) {
				const std::uint32_t bt = hi >= 32 ? B : (B << (32 - hi));
				const std::uint32_t L  = __clz(~bt);
				elem = (nbv == 0 ? 1u : 0u) | ((L & 1u) << 1) | ((__popc(T0) & 1u) << 2)
					 | (((D & fbit) ? 1u : 0u) << 3);
			}
			F.ex0  = ex0;
			F.aux  = esc0;
			F.fbit = fbit;
			F.elem = elem;
			// scan 1: element
			{
				std::uint32_t e1[4] = {elem, 0, 0, 0}, x1[4], t1[4];
				const std::uint32_t id[4] = {kIdent, 0, 0, 0};
				block_scan<1>(e1, x1, t1, id, OpElem(), sc.wpart[buf]);
				F.pre  = x1[0];
				tot[3] = t1[0];
			}
			// word counts under tile hypotheses (e_t = 0, p_t = 0 / 1)
			const std::uint32_t e_w	  = (F.pre >> 1) & 1u;
			const std::uint32_t q_pre = (F.pre >> 2) & 1u;
			const std::uint32_t above = fbit ? ~((fbit << 1) - 1u) : 0u;
			const std::uint32_t exw	  = ex0 ^ ((e_w && (D & fbit)) ? above : 0u);
			auto pk = [&](std::uint32_t X) {
				const std::uint32_t c0 = __popc(X & ~exw), c1 = __popc(X & exw);
				return q_pre ? (c1 | (c0 << 16)) : (c0 | (c1 << 16));
			};
			v[0] = pk(S);
			v[1] = BR ? pk(O) : 0u;
			v[2] = BR ? pk(C) : 0u;
			v[3] = 0;
			const std::uint32_t id[4] = {0, 0, 0, 0};
			std::uint32_t		t2[4];
			block_scan<3>(v, ex, t2, id, OpSum3(), sc.wpart[buf]);
			tot[0] = t2[0];
			tot[1] = t2[1];
			tot[2] = t2[2];
			// the tile's first valid non-backslash byte
			const std::uint32_t have = __ballot_sync(kFull, nbv != 0);
			if (tid == 0)
				sc.fword[buf] = 0xFFFFFFFFu;
			__syncthreads();
			if (have && lane == __ffs(have) - 1)
				atomicMin(&sc.fword[buf], static_cast<std::uint32_t>(tid));
			__syncthreads();
			if (tid == static_cast<int>(sc.fword[buf])) {
				sc.fcls[buf] = ((S & fbit) ? 1u : 0u) | ((O & fbit) ? 2u : 0u) | ((C & fbit) ? 4u : 0u);
				sc.dt[buf]	 = (D & fbit) ? 1u : 0u;
			}
			if (tid == 0 && sc.fword[buf] == 0xFFFFFFFFu) {
				sc.fcls[buf] = 0;
				sc.dt[buf]	 = 0;
			}
		}
		F.off[0] = ex[0];
		F.off[1] = ex[1];
		F.off[2] = ex[2];
		if (tid == 0) {
			sc.tile_cnt[buf][0] = tot[0];
			sc.tile_cnt[buf][1] = tot[1];
			sc.tile_cnt[buf][2] = tot[2];
			sc.tile_elem[buf]	= PATH == kPathNone ? kIdent : tot[3];
		}
		__syncthreads();
		// ---- publish AGG (or INCL for the document's first tile) ----------------------
		if (tid == 0) {
			uint4 d;
			if (PATH == kPathNone) {
				d = make_uint4(tot[0], tot[1], tot[2], 0u);
			} else if (PATH == kPathEscape) {
				const std::uint32_t fcl = sc.fcls[buf];
				// hi counts: the first non-backslash byte's own contribution removed
				d = make_uint4(tot[0] - (fcl & 1u), tot[1] - ((fcl >> 1) & 1u),
							   tot[2] - ((fcl >> 2) & 1u), (tot[3] & 0xFu) | (fcl << 4));
			} else {
				d = make_uint4(tot[0], tot[1], tot[2], tot[3] & 0xFu);
			}
			if (t == 0) {
				std::uint32_t cs, co, cc;
				agg_counts<PATH>(d, init_state, cs, co, cc);
				const std::uint32_t after = PATH == kPathNone ? 0u : apply_fast(tot[3], init_state);
				st128_release(&desc[0], make_uint4(base0[0] + cs, base0[1] + co, base0[2] + cc,
												   kDIncl | (epoch << 8) | after));
			} else {
				d.w |= kDAgg | (epoch << 8);
				st128_release(&desc[t], d);
			}
		}
	};

	// ---------------------------------------------------------- look-back fold ----
	// Loads issued early (before the next tile's phase A); resolved here.
	auto fold = [&](unsigned long long t, uint4 lb) {
		const long long W = t < G ? static_cast<long long>(t) : static_cast<long long>(G);
		bool			mine = tid < W;
		if (mine) {
			const unsigned long long idx = t - 1 - tid;
			std::uint32_t			 spins = 0;
			while (!((lb.w >> 30) != 0 && ((lb.w >> 8) & 0x3FFFFFu) == epoch)) {
				if (++spins > kSpinLimit) {
					record_error(res, kDevErrTimeout);
					sc.failed = 1;
					lb		  = make_uint4(0, 0, 0, kDIncl);
					break;
				}
				if ((spins & 63u) == 0 && aborted(res)) {
					sc.failed = 1;
					lb		  = make_uint4(0, 0, 0, kDIncl);
					break;
				}
				__nanosleep(32);
				lb = ld128_relaxed(&desc[idx]);
			}
		}
		const bool incl = mine && (lb.w >> 30) == 2u;
		if (tid == 0)
			sc.fold_J = static_cast<std::uint32_t>(W);
		__syncthreads();
		const std::uint32_t ib = __ballot_sync(kFull, incl);
		if (ib && lane == __ffs(ib) - 1)
			atomicMin(&sc.fold_J, static_cast<std::uint32_t>(tid));
		__syncthreads();
		const int J = static_cast<int>(sc.fold_J);
		if (tid == J && J < W) {
			sc.incl_state  = lb.w & 3u;
			sc.incl_cnt[0] = lb.x;
			sc.incl_cnt[1] = lb.y;
			sc.incl_cnt[2] = lb.z;
		}
		const int nw = (J + 31) / 32;  // warps holding AGG entries (tid < J)
		std::uint32_t ev = kIdent, excl_rev = kIdent;
		if (warp < nw) {
			ev = (tid < J) ? (lb.w & 0xFu) : kIdent;
			std::uint32_t x = ev;
#pragma unroll
			for (int off = 1; off < 32; off <<= 1) {
				const std::uint32_t o = __shfl_down_sync(kFull, x, off);
				if (lane + off < 32)
					x = compose_fast(o, x);	 // older (higher tid) first
			}
			excl_rev = __shfl_down_sync(kFull, x, 1);
			if (lane == 31)
				excl_rev = kIdent;
			if (lane == 0)
				sc.warp_elem[warp] = x;
		}
		__syncthreads();
		if (tid == 0) {
			std::uint32_t st = (J < W) ? sc.incl_state : init_state;
			for (int w = nw - 1; w >= 0; --w) {
				sc.s_enter[w] = st;
				st			  = apply_fast(sc.warp_elem[w], st);
			}
			sc.in_state = PATH == kPathNone ? 0u : st;
		}
		__syncthreads();
		if (warp < nw) {
			std::uint32_t cs = 0, co = 0, cc = 0;
			if (tid < J) {
				const std::uint32_t st = apply_fast(excl_rev, sc.s_enter[warp]);
				agg_counts<PATH>(lb, st, cs, co, cc);
			}
#pragma unroll
			for (int off = 16; off > 0; off >>= 1) {
				cs += __shfl_xor_sync(kFull, cs, off);
				co += __shfl_xor_sync(kFull, co, off);
				cc += __shfl_xor_sync(kFull, cc, off);
			}
			if (lane == 0) {
				sc.warp_sum[warp][0] = cs;
				sc.warp_sum[warp][1] = co;
				sc.warp_sum[warp][2] = cc;
			}
		}
		__syncthreads();
		if (tid == 0) {
			std::uint32_t b[3] = {base0[0], base0[1], base0[2]};
			if (J < W) {
				b[0] = sc.incl_cnt[0];
				b[1] = sc.incl_cnt[1];
				b[2] = sc.incl_cnt[2];
			}
			for (int w = 0; w < nw; ++w) {
				b[0] += sc.warp_sum[w][0];
				b[1] += sc.warp_sum[w][1];
				b[2] += sc.warp_sum[w][2];
			}
			sc.base[0] = b[0];
			sc.base[1] = b[1];
			sc.base[2] = b[2];
		}
		__syncthreads();
	};

	// ---------------------------------------------------------------- phase B ----
	auto phase_b = [&](unsigned long long k, Front& F) {
		const unsigned long long t	 = tile_of(k);
		const int				 s	 = static_cast<int>(k % kRing);
		const int				 buf = static_cast<int>(k & 1);
		const unsigned char*	 stage = ring + s * kTileBytes;
		const unsigned long long q0	   = t * kTileBytes + 32ull * tid;
		const std::uint32_t		 s_t   = t == 0 ? init_state : sc.in_state;
		const std::uint32_t		 base[3] = {t == 0 ? base0[0] : sc.base[0],
											t == 0 ? base0[1] : sc.base[1],
											t == 0 ? base0[2] : sc.base[2]};
		// publish INCL (the first tile did it in phase A)
		if (tid == 0 && t != 0) {
			uint4 d;
			if (PATH == kPathNone) {
				d = make_uint4(sc.tile_cnt[buf][0], sc.tile_cnt[buf][1], sc.tile_cnt[buf][2], 0u);
			} else if (PATH == kPathEscape) {
				const std::uint32_t fcl = sc.fcls[buf];
				d = make_uint4(sc.tile_cnt[buf][0] - (fcl & 1u), sc.tile_cnt[buf][1] - ((fcl >> 1) & 1u),
							   sc.tile_cnt[buf][2] - ((fcl >> 2) & 1u),
							   (sc.tile_elem[buf] & 0xFu) | (fcl << 4));
			} else {
				d = make_uint4(sc.tile_cnt[buf][0], sc.tile_cnt[buf][1], sc.tile_cnt[buf][2],
							   sc.tile_elem[buf] & 0xFu);
			}
			std::uint32_t cs, co, cc;
			agg_counts<PATH>(d, s_t, cs, co, cc);
			const std::uint32_t after = PATH == kPathNone ? 0u : apply_fast(sc.tile_elem[buf], s_t);
			st128_release(&desc[t], make_uint4(base[0] + cs, base[1] + co, base[2] + cc,
											   kDIncl | (epoch << 8) | after));
		}
		const std::uint32_t vm	 = bit_range(F.lo, F.hi);
		const std::uint32_t e_t	 = s_t & 1u, p_t = (s_t >> 1) & 1u;
		const std::uint32_t st_w = apply_fast(F.pre, s_t);
		const std::uint32_t e_w = st_w & 1u, p_w = (st_w >> 1) & 1u;
		std::uint32_t off[3];
		if (PATH == kPathNone) {
			off[0] = F.off[0];
			off[1] = F.off[1];
			off[2] = F.off[2];
		} else if (PATH == kPathEscape) {
			if (e_t && static_cast<std::uint32_t>(tid) > sc.fword[buf]) {
				const std::uint32_t p2	= p_t ^ sc.dt[buf];
				const std::uint32_t fcl = sc.fcls[buf];
#pragma unroll
				for (int c = 0; c < 3; ++c) {
					const std::uint32_t f = (fcl >> c) & 1u;
					off[c] = half16(F.off[c], p2) - (p2 == 0 ? f : 0u) + (p_t == 0 ? f : 0u);
				}
			} else {
#pragma unroll
				for (int c = 0; c < 3; ++c) off[c] = half16(F.off[c], p_t);
			}
		} else {
#pragma unroll
			for (int c = 0; c < 3; ++c) off[c] = half16(F.off[c], p_t);
		}
		// R3: the masked bitmap of this word
		std::uint32_t mask = 0, last_flag = 0, endstate = 0;
		if (PATH == kPathParity || PATH == kPathDoubled) {
			mask = ((F.ex0 ^ (p_w ? 0xFFFFFFFFu : 0u)) | F.aux) & vm;
			if (F.hi > F.lo && doc_end <= q0 + 32 && doc_end > q0) {
				endstate  = apply_fast(F.elem, st_w);
				last_flag = (F.D >> (F.hi - 1)) & 1u;
			}
		} else if (PATH == kPathEscape) {
			const std::uint32_t fb	  = F.fbit;
			const std::uint32_t above = fb ? ~((fb << 1) - 1u) : 0u;
			const std::uint32_t exw	  = F.ex0 ^ ((e_w && (F.D & fb)) ? above : 0u);
			mask					  = (exw ^ (p_w ? 0xFFFFFFFFu : 0u)) & vm;
			const std::uint32_t esc	  = F.aux ^ (e_w ? fb : 0u);
			if (F.D & esc & ~mask & vm)
				atomicOr(&res->spec_fail, 1u);
			if (F.hi > F.lo && doc_end <= q0 + 32 && doc_end > q0) {
				endstate  = apply_fast(F.elem, st_w);
				last_flag = ((F.D & ~esc) >> (F.hi - 1)) & 1u;
			}
		}
		// end of document / chunk
		if (F.hi > F.lo && doc_end <= q0 + 32 && doc_end > q0) {
			const std::uint32_t unclosed = PATH == kPathNone ? 0u : (((endstate >> 1) & 1u) | last_flag);
			res->unclosed				 = unclosed;
			if (a.carry_out) {
				a.carry_out->fstate		 = endstate;
				a.carry_out->last_delim	 = (F.D >> (F.hi - 1)) & 1u;
				a.carry_out->last_toggle = last_flag;
				a.carry_out->unclosed	 = unclosed;
			}
		}
		if (t == a.ntiles - 1 && tid == 0) {
			std::uint32_t cs, co, cc;
			uint4		  d;
			if (PATH == kPathNone) {
				d = make_uint4(sc.tile_cnt[buf][0], sc.tile_cnt[buf][1], sc.tile_cnt[buf][2], 0u);
			} else if (PATH == kPathEscape) {
				const std::uint32_t fcl = sc.fcls[buf];
				d = make_uint4(sc.tile_cnt[buf][0] - (fcl & 1u), sc.tile_cnt[buf][1] - ((fcl >> 1) & 1u),
							   sc.tile_cnt[buf][2] - ((fcl >> 2) & 1u),
							   (sc.tile_elem[buf] & 0xFu) | (fcl << 4));
			} else {
				d = make_uint4(sc.tile_cnt[buf][0], sc.tile_cnt[buf][1], sc.tile_cnt[buf][2],
							   sc.tile_elem[buf] & 0xFu);
			}
			agg_counts<PATH>(d, s_t, cs, co, cc);
			const unsigned long long ns = static_cast<unsigned long long>(base[0]) + cs;
			const unsigned long long no = static_cast<unsigned long long>(base[1]) + co;
			const unsigned long long nc = static_cast<unsigned long long>(base[2]) + cc;
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
		// R2/R3 select + R5 outputs
		const std::uint32_t sel	 = F.S & ~mask;
		const std::uint32_t selo = F.O & ~mask;
		const std::uint32_t selc = F.C & ~mask;
		unsigned long long	si	 = static_cast<unsigned long long>(base[0]) + off[0];
		const unsigned long long no0 = static_cast<unsigned long long>(base[1]) + off[1];
		const unsigned long long nc0 = static_cast<unsigned long long>(base[2]) + off[2];
		unsigned long long	bi	 = no0 + nc0;
		long long			dep	 = static_cast<long long>(no0) - static_cast<long long>(nc0);
		const unsigned long long pos0 = byte_base + q0 - a.o;
		const unsigned char*	 wb	  = stage + 32 * tid;
		std::uint32_t			 m	  = sel;
		const std::uint32_t		 bm	  = selo | selc;
		while (m) {
			const int j = __ffs(m) - 1;
			m &= m - 1;
			const std::uint32_t pos = static_cast<std::uint32_t>(pos0 + j);
			if (si < a.cap_s) {
				a.pos[si] = pos;
				if (want_chars)
					a.chars[si] = wb[j];
				if (want_pairs)
					a.pair[si] = -1;
			}
			if (BR && ((bm >> j) & 1u)) {
				const bool		op	= (selo >> j) & 1u;
				const long long key = op ? dep : dep - 1;
				dep += op ? 1 : -1;
				if (bi < a.cap_b) {
					a.bpos[bi]	= pos;
					a.bchar[bi] = wb[j];
					a.bsi[bi]	= static_cast<std::uint32_t>(si);
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
		if (want_mask && F.lo < F.hi)
			a.mask[(byte_base + q0 - a.o) >> 5] = mask;
	};

	// ----------------------------------------------------------------- pipeline ----
	Front cur, nxt;
	if (n_mine > 0)
		phase_a(0, cur);
	for (unsigned long long k = 0; k < n_mine; ++k) {
		const unsigned long long t = tile_of(k);
		// look-back loads of tile t (resolved after the next tile's phase A)
		uint4 lb = make_uint4(0, 0, 0, 0);
		const unsigned long long W = t < G ? t : G;
		if (static_cast<unsigned long long>(tid) < W)
			lb = ld128_relaxed(&desc[t - 1 - tid]);
		if (k + 1 < n_mine)
			phase_a(k + 1, nxt);
		if (t > 0)
			fold(t, lb);
		if (sc.failed)
			break;
		phase_b(k, cur);
		__syncthreads();
		if (tid == 0)
			issue(k + kRing);  // ring slot of tile k is free again
		cur = nxt;
	}

	// ---- drain copies still in flight after a failure -------------------------------
	if (tid == 0 && sc.failed) {
		for (unsigned long long k = waited; k < issued; ++k) {
			const int	  s		= static_cast<int>(k % kRing);
			std::uint32_t spins = 0;
			while (!mbar_try_wait(&bars[s], (phase_bits >> s) & 1u) && ++spins < kSpinLimit) {
			}
			phase_bits ^= 1u << s;
		}
	}

	// ---- CTA exit: depth extrema and key histogram ----------------------------------
	if (BR) {
		const long long v0 = warp_min(ext_min_bal), v1 = warp_max(ext_max_bal);
		const long long v2 = warp_min(ext_min_key), v3 = warp_max(ext_max_key);
		const bool		anyk = __any_sync(kFull, any_keys);
		if (lane == 0) {
			sc.wext[0][warp] = v0;
			sc.wext[1][warp] = v1;
			sc.wext[2][warp] = v2;
			sc.wext[3][warp] = v3;
		}
		if (tid == 0)
			sc.any_br = 0;
		__syncthreads();
		if (lane == 0 && anyk)
			atomicOr(&sc.any_br, 1u);
		__syncthreads();
		if (tid == 0 && sc.any_br) {
			long long mn = 0, mx = 0, kn = 0x7FFFFFFFFFFFFFFFll, kx = -0x7FFFFFFFFFFFFFFFll;
			for (int w = 0; w < kWarps; ++w) {
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
			for (int i = tid; i < 2 * kKeyWindow; i += kScanThreads)
				if (khist[i])
					atomicAdd(&a.key_hist[i], khist[i]);
	}
}

#define PARS_INST(P, B) template __global__ void k_scan_fast<P, B>(const ScanArgs);
PARS_INST(kPathNone, false)
PARS_INST(kPathNone, true)
PARS_INST(kPathParity, false)
PARS_INST(kPathParity, true)
PARS_INST(kPathDoubled, false)
PARS_INST(kPathDoubled, true)
PARS_INST(kPathEscape, false)
PARS_INST(kPathEscape, true)
#undef PARS_INST

int scan_fast_smem_bytes() {
	return SmemFast::kBytes;
}

const void* scan_fast_kernel(int path, bool brackets) {
	switch (path * 2 + (brackets ? 1 : 0)) {
		case 0: return reinterpret_cast<const void*>(&k_scan_fast<kPathNone, false>);
		case 1: return reinterpret_cast<const void*>(&k_scan_fast<kPathNone, true>);
		case 2: return reinterpret_cast<const void*>(&k_scan_fast<kPathParity, false>);
		case 3: return reinterpret_cast<const void*>(&k_scan_fast<kPathParity, true>);
		case 4: return reinterpret_cast<const void*>(&k_scan_fast<kPathDoubled, false>);
		case 5: return reinterpret_cast<const void*>(&k_scan_fast<kPathDoubled, true>);
		case 6: return reinterpret_cast<const void*>(&k_scan_fast<kPathEscape, false>);
		default: return reinterpret_cast<const void*>(&k_scan_fast<kPathEscape, true>);
	}
}

}  // namespace pars
