// pars_oracle.cpp — CPU oracle for the pars R1–R6 structural scan.
//
// TEST INFRASTRUCTURE ONLY.  This file is the correctness checker: it is used by
// tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by
// the product path (pars_gb300/ has no reference to it).
//
// It is a plain restatement of the reference CPU backend, driven by the serialized
// scan_plan at run time instead of a compile-time template argument:
//   * R1 classifier  — include/pars/model/classify.hpp:13-55 (build_classifier, cbit)
//   * R3+R4+R5 scan  — include/pars/model/scan.hpp:33-72 (scanner<S>::scan)
//   * R6 pairing     — include/pars/model/nest.hpp:46-92 (pair_brackets<S>)
// plus two values the reference computes internally but does not return:
//   * the per-byte `masked` bit (scan.hpp:45-52), packed 32 bytes per uint32 word;
//   * the per-bracket depth key: open -> bal-1, close -> bal (nest.hpp:72-76).
//
// Plan byte layout (3177 bytes, no padding), identical to pars::scan_plan in
// include/pars/plan.hpp:39-79:
//   [0,8) punctuation  [8,24) brackets{open,close}x8  [24,40) modes{delim,escape}x8
//   [40,44) comments  44 n_punct 45 n_brackets 46 n_modes 47 n_comments
//   [48, 48+8*391) descs; each lex_desc: 0 kind 1 n_states 2 n_classes 3 start
//   4 ok 5 delim 6 escape [7,263) rep_of [263,327) trans[8][8] [327,391) masked[8][8]
//   3176 n_descs
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

namespace {

constexpr std::size_t kPlanBytes = 3177;
constexpr std::size_t kDescBytes = 391;
constexpr std::size_t kDescOff   = 48;

struct Desc {
	std::uint8_t n_states, n_classes, start;
	std::uint8_t rep_of[256];
	std::uint8_t trans[8][8];
	std::uint8_t masked[8][8];
};

struct Plan {
	std::uint8_t punct[8], open[8], close[8], delim[8], escape[8], comment[4];
	int			 n_punct, n_brackets, n_modes, n_comments, n_descs;
	Desc		 desc[8];
	std::uint32_t cls[256];	 // bit0 structural, bit1 open, bit2 close (classify.hpp:13-29)
};

constexpr std::uint32_t kStruct = 1u, kOpen = 2u, kClose = 4u;

bool parse_plan(const std::uint8_t* b, std::uint64_t len, Plan& p) {
	if (!b || len != kPlanBytes)
		return false;
	std::memset(&p, 0, sizeof p);
	p.n_punct	 = b[44];
	p.n_brackets = b[45];
	p.n_modes	 = b[46];
	p.n_comments = b[47];
	p.n_descs	 = b[3176];
	if (p.n_punct > 8 || p.n_brackets > 8 || p.n_modes > 8 || p.n_comments > 4 || p.n_descs > 8)
		return false;
	for (int i = 0; i < 8; ++i) {
		p.punct[i]	= b[i];
		p.open[i]	= b[8 + 2 * i];
		p.close[i]	= b[8 + 2 * i + 1];
		p.delim[i]	= b[24 + 2 * i];
		p.escape[i] = b[24 + 2 * i + 1];
	}
	for (int i = 0; i < 4; ++i) p.comment[i] = b[40 + i];
	for (int d = 0; d < p.n_descs; ++d) {
		const std::uint8_t* q = b + kDescOff + d * kDescBytes;
		Desc&				D = p.desc[d];
		D.n_states			  = q[1];
		D.n_classes			  = q[2];
		D.start				  = q[3];
		if (D.n_states == 0 || D.n_states > 8 || D.n_classes == 0 || D.n_classes > 8
			|| D.start >= D.n_states)
			return false;
		std::memcpy(D.rep_of, q + 7, 256);
		std::memcpy(D.trans, q + 263, 64);
		std::memcpy(D.masked, q + 327, 64);
		for (int c = 0; c < 256; ++c)
			if (D.rep_of[c] >= D.n_classes)
				return false;
		for (int s = 0; s < D.n_states; ++s)
			for (int c = 0; c < D.n_classes; ++c)
				if (D.trans[s][c] >= D.n_states)
					return false;
	}
	// classify.hpp:39-55: punctuation -> structural; brackets -> structural|open/close.
	for (int i = 0; i < p.n_punct; ++i) p.cls[p.punct[i]] |= kStruct;
	for (int i = 0; i < p.n_brackets; ++i) {
		p.cls[p.open[i]] |= kStruct | kOpen;
		p.cls[p.close[i]] |= kStruct | kClose;
	}
	return true;
}

// nest.hpp:24-44
bool is_open(const Plan& p, std::uint8_t c) {
	for (int i = 0; i < p.n_brackets; ++i)
		if (p.open[i] == c)
			return true;
	return false;
}

bool is_close(const Plan& p, std::uint8_t c) {
	for (int i = 0; i < p.n_brackets; ++i)
		if (p.close[i] == c)
			return true;
	return false;
}

bool match(const Plan& p, std::uint8_t o, std::uint8_t c) {
	for (int i = 0; i < p.n_brackets; ++i)
		if (p.open[i] == o)
			return p.close[i] == c;
	return false;
}

}  // namespace

extern "C" {

// Size of the plan POD this oracle understands.
std::uint64_t oracle_plan_bytes() {
	return kPlanBytes;
}

// R3+R4+R5 (scan.hpp:33-72).  Output arrays may be null when their capacity is 0;
// entries past a capacity are counted but not written.  `mask_words` (optional)
// receives ceil(n/32) words, bit j of word w = masked(byte 32w+j).
// counts[0]=n_struct counts[1]=n_brackets counts[2]=unclosed_mode.
// Returns 0, or -1 for a malformed plan.
int oracle_scan(
	const std::uint8_t* plan, std::uint64_t plan_len, const std::uint8_t* in, std::uint64_t n,
	std::uint32_t* pos, std::uint8_t* chars, std::uint64_t cap_struct, std::uint32_t* bpos,
	std::uint8_t* bchar, std::uint64_t cap_br, std::uint32_t* mask_words, std::uint64_t* counts
) {
	Plan P;
	if (!parse_plan(plan, plan_len, P))
		return -1;
	std::uint8_t st[8];
	for (int d = 0; d < P.n_descs; ++d) st[d] = P.desc[d].start;
	if (mask_words)
		std::memset(mask_words, 0, ((n + 31) / 32) * 4);
	std::uint64_t ns = 0, nb = 0;
	for (std::uint64_t i = 0; i < n; ++i) {
		const std::uint8_t c = in[i];
		bool			   m = false;
		for (int d = 0; d < P.n_descs; ++d) {
			const Desc&		   D  = P.desc[d];
			const std::uint8_t cl = D.rep_of[c];
			if (D.masked[st[d]][cl])
				m = true;
			st[d] = D.trans[st[d]][cl];
		}
		if (m) {
			if (mask_words)
				mask_words[i >> 5] |= 1u << (i & 31);
			continue;
		}
		const std::uint32_t k = P.cls[c];
		if (k & kStruct) {
			if (ns < cap_struct) {
				if (pos)
					pos[ns] = static_cast<std::uint32_t>(i);
				if (chars)
					chars[ns] = c;
			}
			++ns;
			if (k & (kOpen | kClose)) {
				if (nb < cap_br) {
					if (bpos)
						bpos[nb] = static_cast<std::uint32_t>(i);
					if (bchar)
						bchar[nb] = c;
				}
				++nb;
			}
		}
	}
	bool unclosed = false;
	for (int d = 0; d < P.n_descs; ++d)
		if (st[d] != P.desc[d].start)
			unclosed = true;
	counts[0] = ns;
	counts[1] = nb;
	counts[2] = unclosed ? 1 : 0;
	return 0;
}

// R6 (nest.hpp:46-92).  pair[i] is the partner's bracket index or -1 (bracket-index
// space, like the reference); depth[i] is the sort key (open: bal-1, close: bal).
// flags[0]=balanced flags[1]=well_formed flags[2]=max_depth.
int oracle_pair(
	const std::uint8_t* plan, std::uint64_t plan_len, const std::uint8_t* bchar, std::uint64_t n,
	std::int32_t* pair, std::int32_t* depth, std::int32_t* flags
) {
	Plan P;
	if (!parse_plan(plan, plan_len, P))
		return -1;
	flags[0] = 1;
	flags[1] = 1;
	flags[2] = 0;
	for (std::uint64_t i = 0; i < n; ++i) pair[i] = -1;
	if (n == 0)
		return 0;
	std::vector<std::int32_t> bal(n), key(n);
	std::vector<std::uint8_t> op(n);
	int						  run = 0;
	for (std::uint64_t i = 0; i < n; ++i) {
		op[i] = is_open(P, bchar[i]) ? 1 : 0;
		run += op[i] ? 1 : -1;
		bal[i] = run;
		key[i] = op[i] ? run - 1 : run;
		if (depth)
			depth[i] = key[i];
	}
	int max_depth = 0, min_bal = 0;
	for (std::uint64_t i = 0; i < n; ++i) {
		max_depth = std::max(max_depth, bal[i]);
		min_bal	  = std::min(min_bal, bal[i]);
	}
	const bool balanced = (min_bal >= 0) && (bal[n - 1] == 0);
	bool	   wf		= true;
	std::vector<std::int32_t> order(n);
	std::iota(order.begin(), order.end(), 0);
	std::stable_sort(order.begin(), order.end(), [&](std::int32_t a, std::int32_t b) {
		return key[a] < key[b];
	});
	for (std::uint64_t k = 0; k + 1 < n; k += 2) {
		const std::int32_t a = order[k], b = order[k + 1];
		if (op[a] && is_close(P, bchar[b]) && match(P, bchar[a], bchar[b])) {
			pair[a] = b;
			pair[b] = a;
		} else {
			wf = false;
		}
	}
	if (n % 2 != 0)
		wf = false;
	flags[0] = balanced ? 1 : 0;
	flags[1] = (wf && balanced) ? 1 : 0;
	flags[2] = max_depth;
	return 0;
}

// Runs scan then pair over `in` `iters` times into caller scratch and returns the
// mean wall seconds per iteration (used only as the CPU baseline timing).
double oracle_time_scan_pair(
	const std::uint8_t* plan, std::uint64_t plan_len, const std::uint8_t* in, std::uint64_t n,
	int iters, std::uint64_t* counts_out
) {
	Plan P;
	if (!parse_plan(plan, plan_len, P) || iters <= 0)
		return -1.0;
	std::vector<std::uint32_t> pos(n), bpos(n);
	std::vector<std::uint8_t>  chars(n), bchar(n);
	std::vector<std::int32_t>  pair(n), depth(n);
	std::uint64_t			   counts[3] = {0, 0, 0};
	std::int32_t			   flags[3];
	const auto				   t0 = std::chrono::steady_clock::now();
	for (int it = 0; it < iters; ++it) {
		oracle_scan(
			plan, plan_len, in, n, pos.data(), chars.data(), n, bpos.data(), bchar.data(), n,
			nullptr, counts
		);
		oracle_pair(plan, plan_len, bchar.data(), counts[1], pair.data(), depth.data(), flags);
	}
	const auto t1 = std::chrono::steady_clock::now();
	if (counts_out) {
		counts_out[0] = counts[0];
		counts_out[1] = counts[1];
		counts_out[2] = counts[2];
	}
	return std::chrono::duration<double>(t1 - t0).count() / iters;
}

// Runs scan then pair over every document of a batch (`offsets`: ndocs + 1 byte
// offsets into `in`), `iters` times, spread over `threads` host threads that take
// documents one at a time from a shared counter, and returns the mean wall seconds
// per pass over the batch (the CPU baseline of the batched workload: the reference
// scans a document sequentially, so a batch spreads documents over cores).
// counts_out = {structurals, brackets} summed over the documents of one pass.
double oracle_time_batch(
	const std::uint8_t* plan, std::uint64_t plan_len, const std::uint8_t* in,
	const std::uint64_t* offsets, std::uint64_t ndocs, int threads, int iters,
	std::uint64_t* counts_out
) {
	Plan P;
	if (!parse_plan(plan, plan_len, P) || iters <= 0 || threads <= 0 || !offsets)
		return -1.0;
	for (std::uint64_t d = 0; d < ndocs; ++d)
		if (offsets[d + 1] < offsets[d])
			return -1.0;
	std::atomic<std::uint64_t> next {0}, n_struct {0}, n_brackets {0};
	auto work = [&]() {
		std::vector<std::uint32_t> pos, bpos;
		std::vector<std::uint8_t>  chars, bchar;
		std::vector<std::int32_t>  pair, depth;
		std::uint64_t			   ns = 0, nb = 0;
		for (;;) {
			const std::uint64_t d = next.fetch_add(1, std::memory_order_relaxed);
			if (d >= ndocs)
				break;
			const std::uint64_t n = offsets[d + 1] - offsets[d];
			if (pos.size() < n) {
				pos.resize(n);
				bpos.resize(n);
				chars.resize(n);
				bchar.resize(n);
				pair.resize(n);
				depth.resize(n);
			}
			std::uint64_t counts[3] = {0, 0, 0};
			std::int32_t  flags[3];
			oracle_scan(
				plan, plan_len, in + offsets[d], n, pos.data(), chars.data(), n, bpos.data(),
				bchar.data(), n, nullptr, counts
			);
			oracle_pair(plan, plan_len, bchar.data(), counts[1], pair.data(), depth.data(), flags);
			ns += counts[0];
			nb += counts[1];
		}
		n_struct += ns;
		n_brackets += nb;
	};
	const auto t0 = std::chrono::steady_clock::now();
	for (int it = 0; it < iters; ++it) {
		next	   = 0;
		n_struct   = 0;
		n_brackets = 0;
		std::vector<std::thread> pool;
		for (int t = 1; t < threads; ++t) pool.emplace_back(work);
		work();
		for (auto& th : pool) th.join();
	}
	const auto t1 = std::chrono::steady_clock::now();
	if (counts_out) {
		counts_out[0] = n_struct;
		counts_out[1] = n_brackets;
	}
	return std::chrono::duration<double>(t1 - t0).count() / iters;
}

}  // extern "C"
