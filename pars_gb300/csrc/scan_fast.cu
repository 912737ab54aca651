// scan_fast.cu — fused R1..R5 single-pass scan for plans with at most one lexical
// descriptor of a recognised shape (none / quote parity / doubled delimiter /
// prefix escape): the JSON and CSV grammars and their relatives.
//
// Schedule.  A cooperative (all CTAs co-resident) persistent grid of G CTAs walks
// the input in 16 KiB tiles with a static schedule: CTA b owns tiles b, b+G, ...
// Each CTA keeps three tiles in a shared-memory ring (1-D TMA bulk copies that
// complete on mbarriers) and software-pipelines two of them:
//
//     issue look-back loads for tile k
//     phase A(k+1): classify, block scans, publish AGG(k+1)
//     fold the look-back of tile k, publish INCL(k)
//     phase B(k): resolve masks, write offsets / brackets / depth keys
//
// so the look-back's L2 round trip overlaps the classification of the next tile,
// and every predecessor a tile waits for has (in steady state) already published.
//
// Look-back words (128-bit, single-copy atomic), two per tile:
//   AGG[t] : per-class counts of tile t under both in-string hypotheses (u16
//            halves), its automaton element, and (escape path) the class bits of
//            the tile's first non-backslash byte;
//   INCL[t]: the state after tile t and cumulative counts (u32 each).
//   w[31:30] flag, w[29:8] epoch of the launch, w[7:0] element / state bits.
// A tile folds AGG[t-W+1 .. t-1] onto INCL[t-W] with W = min(t, G): tile t-G is
// this CTA's previous tile (its INCL is published) and tile 0 publishes INCL first.
//
// R1 classification: a per-lane replicated [256][32] table in shared memory with a
// 256-byte row stride, 64 KiB-aligned in the shared window, so the address of the
// entry for byte k of a register is one byte permute (byte k -> address bits
// 8..15); 8 lookups are summed with shifts and a 4x4 byte transpose gives the
// structural / open / close / delimiter planes as 32-bit masks.
//
// Reference semantics: include/pars/model/scan.hpp:33-72 and nest.hpp:55-76
// (scan.cu holds the generic descriptor kernel that runs every other plan).
#include <cuda_runtime.h>

#include "fast_common.cuh"

namespace pars {

using namespace scan_detail;

namespace {

constexpr int			kWarps = kScanThreads / 32;

struct FastScratch {
	std::uint32_t wpart[2][kWarps + 1][4];	// block-scan partials (+ total), per tile in flight
	uint4		  agg[2];					// AGG payload of the tile (flag/epoch bits clear)
	std::uint32_t tile_elem[2];
	std::uint32_t fword[2];
	std::uint32_t fcls[2];
	std::uint32_t dt[2];
	// look-back fold result
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
	std::uint32_t vm;
};

// Dynamic shared memory: [ring 3 x 16 KiB][scratch][key histogram][pad][table 64 KiB]
// The table must start on a 64 KiB boundary of the shared window; the pad absorbs
// wherever the dynamic window begins.
struct SmemFast {
	static constexpr int kStage	  = 0;
	static constexpr int kBars	  = kStage + kRing * kTileBytes;
	static constexpr int kScratch = kBars + 64;
	static constexpr int kHist	  = (kScratch + static_cast<int>(sizeof(FastScratch)) + 127) & ~127;
	static constexpr int kLowEnd  = kHist + 2 * kKeyWindow * 4;
	static constexpr int kTblBytes = 256 * 256;
	static constexpr int kBytes	  = kLowEnd + 65536 + kTblBytes;
};

// ---- block-wide exclusive scan of up to 4 u32 lanes (two __syncthreads) ----------
struct NoHook {
	__device__ __forceinline__ void operator()() const {}
};

template<int N, class Op, class Hook = NoHook>
__device__ __forceinline__ void block_scan(std::uint32_t (&v)[4], std::uint32_t (&excl)[4],
										   std::uint32_t (&total)[4], const std::uint32_t (&ident)[4],
										   Op op, std::uint32_t (*wpart)[4], Hook hook = Hook()) {
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
			op(y, x);
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
	hook();
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
	unsigned char* ring = smem + SmemFast::kStage;
	std::uint64_t* bars = reinterpret_cast<std::uint64_t*>(smem + SmemFast::kBars);
	FastScratch&   sc	= *reinterpret_cast<FastScratch*>(smem + SmemFast::kScratch);
	unsigned int*  khist = reinterpret_cast<unsigned int*>(smem + SmemFast::kHist);
	// 64 KiB-aligned table (window address)
	const std::uint32_t win0	= smem_addr(smem);
	const std::uint32_t tbl_win = (win0 + SmemFast::kLowEnd + 0xFFFFu) & ~0xFFFFu;
	std::uint32_t* tbl = reinterpret_cast<std::uint32_t*>(smem + (tbl_win - win0));

	const int			tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const DevPlan*		P	= a.plan;
	DevResult*			res = a.res;
	std::uint64_t*		d_agg  = static_cast<std::uint64_t*>(a.tiles);	// AGG words, planes [3][ntiles]
	std::uint64_t*		d_incl = d_agg + 3 * a.ntiles;					// INCL words, planes [3][ntiles]
	const std::uint64_t nt	   = a.ntiles;
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
	const std::uint32_t escape_rep = P->escape_rep;
	const std::uint8_t	delim	   = P->delim;
	const bool			want_pairs = (a.flags & 1u) != 0;
	const bool			want_chars = (a.flags & 4u) != 0;
	const bool			want_mask  = (a.flags & 8u) != 0 && a.mask;
	const std::uint32_t cap_s = a.cap_s > 0xFFFFFFFFull ? 0xFFFFFFFFu : static_cast<std::uint32_t>(a.cap_s);
	const std::uint32_t cap_b = a.cap_b > 0xFFFFFFFFull ? 0xFFFFFFFFu : static_cast<std::uint32_t>(a.cap_b);

	for (int i = tid; i < 256 * 32; i += kScanThreads) tbl[(i >> 5) * 64 + (i & 31)] = P->cls[i >> 5];
	if (BR)
		for (int i = tid; i < 2 * kKeyWindow; i += kScanThreads) khist[i] = 0;
	if (tid == 0) {
		for (int s = 0; s < kRing; ++s) mbar_init(&bars[s], 1);
		fence_barrier_init();
		sc.failed = 0;
		if (tbl_win + SmemFast::kTblBytes > win0 + SmemFast::kBytes) {
			record_error(res, kDevErrTimeout);	// layout impossible: report, do nothing
			sc.failed = 1;
		}
	}
	__syncthreads();
	if (sc.failed)
		return;

	const std::uint32_t my_first = blockIdx.x;
	const std::uint32_t n_mine	 = my_first < ntiles ? (ntiles - 1 - my_first) / G + 1 : 0u;
	auto tile_of = [&](std::uint32_t k) { return my_first + k * G; };
	std::uint32_t issued = 0, waited = 0;  // tid 0: copies started / consumed
	auto issue = [&](std::uint32_t k) {
		if (k >= n_mine)
			return;
		issued = k + 1;
		const int				 s	   = static_cast<int>(k % kRing);
		const unsigned long long off   = static_cast<unsigned long long>(tile_of(k)) * kTileBytes;
		unsigned long long		 bytes = a.copy_end - off;
		if (bytes > kTileBytes)
			bytes = kTileBytes;
		mbar_arrive_expect_tx(&bars[s], static_cast<std::uint32_t>(bytes));
		bulk_g2s(ring + s * kTileBytes, a.base + off, static_cast<std::uint32_t>(bytes), &bars[s]);
	};
	if (tid == 0)
		for (std::uint32_t k = 0; k < kRing; ++k) issue(k);

	const std::uint32_t tbl_lane = tbl_win + 4u * lane;
	const std::uint32_t sw		 = (tid >> 2) & 1u;	 // which 16-byte half this thread reads first
	const std::uint32_t selA	 = sw ? 0x1054u : 0x5410u;
	const std::uint32_t selB	 = sw ? 0x3276u : 0x7632u;
	std::uint32_t		phase_bits = 0;
	long long ext_min_bal = 0, ext_max_bal = 0;
	long long ext_min_key = 0x7FFFFFFFFFFFFFFFll, ext_max_key = -0x7FFFFFFFFFFFFFFFll;
	bool	  any_keys = false;

	// ---------------------------------------------------------------- phase A ----
	auto phase_a = [&](std::uint32_t k, Front& F) {
		const std::uint32_t t	= tile_of(k);
		// every thread finished phase B of tile k-2 before this tile's first block
		// barrier: tid 0 then reuses that ring slot for tile k+1
		auto refill = [&]() {
			if (tid == 0 && k >= 2)
				issue(k + 1);
		};
		const int			s	= static_cast<int>(k % kRing);
		const int			buf = static_cast<int>(k & 1);
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
		const unsigned long long q0	   = static_cast<unsigned long long>(t) * kTileBytes + 32u * tid;
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
			const uint4* p = reinterpret_cast<const uint4*>(stage + 32 * tid);
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
		F.S	   = S;
		F.O	   = O;
		F.C	   = C;
		F.D	   = D;
		F.aux  = 0;
		F.fbit = 0;
		F.ex0  = 0;
		std::uint32_t v[4], ex[4], tot[4];
		if (PATH == kPathNone) {
			v[0] = __popc(S);
			v[1] = BR ? __popc(O) : 0u;
			v[2] = BR ? __popc(C) : 0u;
			v[3] = 0;
			const std::uint32_t id[4] = {0, 0, 0, 0};
			if (BR)
				block_scan<3>(v, ex, tot, id, OpSum3(), sc.wpart[buf], refill);
			else
				block_scan<1>(v, ex, tot, id, OpSum3(), sc.wpart[buf], refill);
			if (!BR) {
				ex[1] = ex[2] = tot[1] = tot[2] = 0;
			}
			F.pre  = kIdent;
			F.elem = kIdent;
			tot[3] = kIdent;
		} else if (PATH == kPathParity || PATH == kPathDoubled) {
			const std::uint32_t ex0 = prefix_xor32(D) ^ D;
			std::uint32_t		dd	= 0;
			if (PATH == kPathDoubled) {
				// was the byte before each byte a delimiter?
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
			v[1] = __popc(D) & 1u;
			if (BR) {
				v[2] = __popc(O & ~m0) | (__popc(O & ~m1) << 16);
				v[3] = __popc(C & ~m0) | (__popc(C & ~m1) << 16);
			} else {
				v[2] = v[3] = 0;
			}
			std::uint32_t		x[4], tt[4];
			const std::uint32_t id[4] = {0, 0, 0, 0};
			if (BR)
				block_scan<4>(v, x, tt, id, OpParity(), sc.wpart[buf], refill);
			else
				block_scan<2>(v, x, tt, id, OpParity(), sc.wpart[buf], refill);
			ex[0]  = x[0];
			ex[1]  = BR ? x[2] : 0u;
			ex[2]  = BR ? x[3] : 0u;
			tot[0] = tt[0];
			tot[1] = BR ? tt[2] : 0u;
			tot[2] = BR ? tt[3] : 0u;
			tot[3] = 1u | (tt[1] << 2);	 // tile element
			F.ex0  = ex0;
			F.aux  = dd;
			F.pre  = 1u | (x[1] << 2);
			F.elem = 1u | ((__popc(D) & 1u) << 2);
		} else {  // kPathEscape
			const std::uint32_t B	 = eq_mask32(r, escape_rep);
			// the halves of r may be swapped: restore byte order of the escape mask
			const std::uint32_t Bo	 = (sw ? __byte_perm(B, 0, 0x1032u) : B) & vm;
			const std::uint32_t runs = Bo & ~(Bo << 1);
			const std::uint32_t ee	 = (Bo + (runs & 0x55555555u)) & ~Bo;
			const std::uint32_t eo	 = (Bo + (runs & 0xAAAAAAAAu)) & ~Bo;
			const std::uint32_t esc0 = (ee & 0xAAAAAAAAu) | (eo & 0x55555555u);
			const std::uint32_t nbv	 = ~Bo & vm;
			const std::uint32_t fbit = nbv & (0u - nbv);
			const std::uint32_t T0	 = D & ~esc0;
			const std::uint32_t ex0	 = prefix_xor32(T0) ^ T0;
			std::uint32_t		elem = kIdent;
			if (vm != 0) {
				const std::uint32_t bt = hi >= 32 ? Bo : (Bo << (32 - hi));
				const std::uint32_t L  = __clz(~bt);
				elem = (nbv == 0 ? 1u : 0u) | ((L & 1u) << 1) | ((__popc(T0) & 1u) << 2)
					 | (((D & fbit) ? 1u : 0u) << 3);
			}
			F.ex0  = ex0;
			F.aux  = esc0;
			F.fbit = fbit;
			F.elem = elem;
			{
				std::uint32_t		e1[4] = {elem, 0, 0, 0}, x1[4], t1[4];
				const std::uint32_t id[4] = {kIdent, 0, 0, 0};
				block_scan<1>(e1, x1, t1, id, OpElem(), sc.wpart[buf], refill);
				F.pre  = x1[0];
				tot[3] = t1[0];
			}
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
			if (BR)
				block_scan<3>(v, ex, t2, id, OpSum3(), sc.wpart[buf]);
			else
				block_scan<1>(v, ex, t2, id, OpSum3(), sc.wpart[buf]);
			tot[0] = t2[0];
			tot[1] = BR ? t2[1] : 0u;
			tot[2] = BR ? t2[2] : 0u;
			if (!BR)
				ex[1] = ex[2] = 0;
			// the tile's first valid non-backslash byte (its owner records class / quote)
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
			__syncthreads();
		}
		F.off[0] = ex[0];
		F.off[1] = ex[1];
		F.off[2] = ex[2];
		// ---- publish AGG (or, for the document's first tile, INCL) -----------------
		if (tid == 0) {
			uint4 d;
			if (PATH == kPathNone) {
				d = make_uint4(tot[0], tot[1], tot[2], 0u);
			} else if (PATH == kPathEscape) {
				const std::uint32_t fcl = sc.fcls[buf];
				d = make_uint4(tot[0] - (fcl & 1u), tot[1] - ((fcl >> 1) & 1u),
							   tot[2] - ((fcl >> 2) & 1u), (tot[3] & 0xFu) | (fcl << 4));
			} else {
				d = make_uint4(tot[0], tot[1], tot[2], tot[3] & 0xFu);
			}
			sc.agg[buf]		  = d;
			sc.tile_elem[buf] = tot[3];
			if (t == 0) {
				std::uint32_t cs, co, cc;
				agg_counts<PATH>(d, init_state, cs, co, cc);
				const std::uint32_t after = PATH == kPathNone ? 0u : apply_fast(tot[3], init_state);
				st_desc(d_incl, nt, 0, make_uint4(base0[0] + cs, base0[1] + co, base0[2] + cc,
												  kDIncl | (epoch << 8) | after));
			} else {
				d.w |= kDAgg | (epoch << 8);
				st_desc(d_agg, nt, t, d);
			}
		}
	};

	// ---------------------------------------------------------- look-back fold ----
	// Warp 0 holds the look-back words of tile t: lane l, slot i covers distance
	// j = l*kLB + i (j = 0 is tile t-1).  Slots j < W-1 are AGG words, j == W-1 is
	// the INCL word of tile t-W (W = min(t, G) <= 32*kLB).  The loads are issued
	// before the next tile's phase A and folded here; one block barrier follows.
	auto load_lb = [&](std::uint32_t t, uint4 (&lbv)[kLB]) {
		const std::uint32_t W = t < G ? t : G;
#pragma unroll
		for (int i = 0; i < kLB; ++i) {
			const std::uint32_t j = static_cast<std::uint32_t>(lane) * kLB + i;
			lbv[i]				  = make_uint4(0, 0, 0, 0);
			if (j + 1 < W)
				lbv[i] = ld_desc(d_agg, nt, t - 1 - j);
			else if (j + 1 == W)
				lbv[i] = ld_desc(d_incl, nt, t - W);
		}
	};
	auto fold = [&](std::uint32_t t, uint4 (&lbv)[kLB]) {
		if (warp == 0) {
			const std::uint32_t W	 = t < G ? t : G;
			bool				bad	 = false;
#pragma unroll
			for (int i = 0; i < kLB; ++i) {
				const std::uint32_t j = static_cast<std::uint32_t>(lane) * kLB + i;
				if (j < W) {
					const bool			incl_slot = (j + 1 == W);
					const std::uint64_t* src	  = incl_slot ? d_incl : d_agg;
					const std::uint64_t	 idx	  = incl_slot ? t - W : t - 1 - j;
					const std::uint32_t want	  = incl_slot ? 2u : 1u;
					std::uint32_t		spins	  = 0;
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
						lbv[i] = ld_desc(src, nt, idx);
					}
				}
			}
			if (__any_sync(kFull, bad)) {
				if (lane == 0)
					sc.failed = 1;
			} else {
				// the INCL word
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
				// this lane's AGG elements, oldest first
				std::uint32_t E = kIdent;
#pragma unroll
				for (int i = kLB - 1; i >= 0; --i)
					if (static_cast<std::uint32_t>(lane) * kLB + i + 1 < W)
						E = compose_fast(E, lbv[i].w & 0xFu);
				std::uint32_t x = E;
#pragma unroll
				for (int off = 1; off < 32; off <<= 1) {
					const std::uint32_t o = __shfl_down_sync(kFull, x, off);
					if (lane + off < 32)
						x = compose_fast(o, x);	 // older (higher lane) first
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
				if (lane == 0) {
					sc.in_state = st;  // lane 0 ends with the newest tile (t-1)
					sc.base[0]	= c_incl[0] + cs;
					sc.base[1]	= c_incl[1] + co;
					sc.base[2]	= c_incl[2] + cc;
				}
			}
		}
		__syncthreads();
	};

	// ---------------------------------------------------------------- phase B ----
	auto phase_b = [&](std::uint32_t k, const Front& F) {
		const std::uint32_t		 t	   = tile_of(k);
		const int				 s	   = static_cast<int>(k % kRing);
		const int				 buf   = static_cast<int>(k & 1);
		const unsigned char*	 stage = ring + s * kTileBytes;
		const unsigned long long q0	   = static_cast<unsigned long long>(t) * kTileBytes + 32u * tid;
		const std::uint32_t		 s_t   = t == 0 ? init_state : sc.in_state;
		const std::uint32_t base[3] = {t == 0 ? base0[0] : sc.base[0], t == 0 ? base0[1] : sc.base[1],
									   t == 0 ? base0[2] : sc.base[2]};
		if (tid == 0 && t != 0) {
			std::uint32_t cs, co, cc;
			agg_counts<PATH>(sc.agg[buf], s_t, cs, co, cc);
			const std::uint32_t after = PATH == kPathNone ? 0u : apply_fast(sc.tile_elem[buf], s_t);
			st_desc(d_incl, nt, t, make_uint4(base[0] + cs, base[1] + co, base[2] + cc,
											  kDIncl | (epoch << 8) | after));
		}
		const std::uint32_t vm	 = F.vm;
		const std::uint32_t e_t	 = s_t & 1u, p_t = (s_t >> 1) & 1u;
		const std::uint32_t st_w = apply_fast(F.pre, s_t);
		const std::uint32_t e_w = st_w & 1u, p_w = (st_w >> 1) & 1u;
		std::uint32_t		off[3];
		if (PATH == kPathNone) {
			off[0] = F.off[0];
			off[1] = F.off[1];
			off[2] = F.off[2];
		} else if (PATH == kPathEscape && e_t && static_cast<std::uint32_t>(tid) > sc.fword[buf]) {
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
		// R3: masked bitmap of this word
		std::uint32_t mask = 0, esc = 0;
		if (PATH == kPathParity || PATH == kPathDoubled) {
			mask = ((F.ex0 ^ (p_w ? 0xFFFFFFFFu : 0u)) | F.aux) & vm;
		} else if (PATH == kPathEscape) {
			const std::uint32_t fb	  = F.fbit;
			const std::uint32_t above = fb ? ~((fb << 1) - 1u) : 0u;
			const std::uint32_t exw	  = F.ex0 ^ ((e_w && (F.D & fb)) ? above : 0u);
			mask					  = (exw ^ (p_w ? 0xFFFFFFFFu : 0u)) & vm;
			esc						  = F.aux ^ (e_w ? fb : 0u);
			if (F.D & esc & ~mask)
				atomicOr(&res->spec_fail, 1u);
		}
		// end of document / chunk: the thread holding the last byte
		if (vm != 0 && doc_end <= q0 + 32 && doc_end > q0) {
			const int			hi		  = static_cast<int>(doc_end - q0);
			const std::uint32_t endstate  = PATH == kPathNone ? 0u : apply_fast(F.elem, st_w);
			const std::uint32_t last_flag = PATH == kPathEscape ? (((F.D & ~esc) >> (hi - 1)) & 1u)
																: ((F.D >> (hi - 1)) & 1u);
			const std::uint32_t unclosed = PATH == kPathNone ? 0u : (((endstate >> 1) & 1u) | last_flag);
			res->unclosed				 = unclosed;
			if (a.carry_out) {
				a.carry_out->fstate		 = endstate;
				a.carry_out->last_delim	 = (F.D >> (hi - 1)) & 1u;
				a.carry_out->last_toggle = last_flag;
				a.carry_out->unclosed	 = unclosed;
			}
		}
		if (t == ntiles - 1 && tid == 0) {
			std::uint32_t cs, co, cc;
			agg_counts<PATH>(sc.agg[buf], s_t, cs, co, cc);
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
		std::uint32_t		m	 = F.S & ~mask;
		const std::uint32_t selo = BR ? (F.O & ~mask) : 0u;
		const std::uint32_t selc = BR ? (F.C & ~mask) : 0u;
		std::uint32_t		si	 = base[0] + off[0];
		const std::uint32_t pos0 = byte_base + static_cast<std::uint32_t>(q0 - a.o);
		const unsigned char* wb	 = stage + 32 * tid;
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
			const std::uint32_t no0 = base[1] + off[1];
			const std::uint32_t nc0 = base[2] + off[2];
			std::uint32_t		bi	= no0 + nc0;
			long long			dep = static_cast<long long>(no0) - static_cast<long long>(nc0);
			const std::uint32_t bm	= selo | selc;
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
	};

	// ----------------------------------------------------------------- pipeline ----
	auto step = [&](std::uint32_t k, Front& Fc, Front& Fn) -> bool {
		const std::uint32_t t = tile_of(k);
		uint4				lbv[kLB];
		if (warp == 0 && t > 0)
			load_lb(t, lbv);
		if (k + 1 < n_mine)
			phase_a(k + 1, Fn);
		if (t > 0)
			fold(t, lbv);
		if (sc.failed)
			return false;
		phase_b(k, Fc);
		return true;
	};
	Front f0, f1;
	if (n_mine > 0)
		phase_a(0, f0);
	for (std::uint32_t k = 0; k < n_mine; k += 2) {
		if (!step(k, f0, f1))
			break;
		if (k + 1 < n_mine && !step(k + 1, f1, f0))
			break;
	}
	__syncthreads();

	// ---- drain copies still in flight after a failure -------------------------------
	if (tid == 0 && sc.failed) {
		for (std::uint32_t k = waited; k < issued; ++k) {
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

int scan_fast_max_grid() {
	return 32 * kLB;
}

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
