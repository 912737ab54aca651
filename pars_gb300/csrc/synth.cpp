// synth.cpp — seeded synthetic documents for the pars structural-scan workloads.
//
// Host-only C++ (no CUDA), built into libpars_synth.so.  Every generator is a pure
// function of (seed, parameters): the same call yields the same bytes on x86 and
// Arm.  The PRNG is xoshiro256** seeded through splitmix64.
//
//   pars_synth_json  — random JSON value tree (objects / arrays / scalars) with a
//                      byte budget; containers still open at the budget are closed,
//                      so the output is always one well-formed top-level array.
//   pars_synth_csv   — RFC-4180-style CSV with LF records and quoted fields.
//   pars_synth_config — TOML / C-like / INI / XML documents mixing every lexical
//                      mode of the grammar with structural bytes in and out of them.
//   pars_synth_alpha — uniform random bytes over an alphabet (adversarial inputs).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Rng {
	std::uint64_t s[4];

	explicit Rng(std::uint64_t seed) {
		std::uint64_t x = seed;
		for (auto& v : s) {
			x += 0x9E3779B97F4A7C15ull;
			std::uint64_t z = x;
			z				= (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
			z				= (z ^ (z >> 27)) * 0x94D049BB133111EBull;
			v				= z ^ (z >> 31);
		}
	}

	static std::uint64_t rotl(std::uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

	std::uint64_t next() {
		const std::uint64_t r = rotl(s[1] * 5, 7) * 9;
		const std::uint64_t t = s[1] << 17;
		s[2] ^= s[0];
		s[3] ^= s[1];
		s[1] ^= s[2];
		s[0] ^= s[3];
		s[2] ^= t;
		s[3] = rotl(s[3], 45);
		return r;
	}

	// uniform in [lo, hi]
	std::uint64_t range(std::uint64_t lo, std::uint64_t hi) { return lo + next() % (hi - lo + 1); }

	double unit() { return (next() >> 11) * (1.0 / 9007199254740992.0); }

	bool chance(double p) { return unit() < p; }
};

struct Out {
	std::uint8_t* p;
	std::uint64_t cap, n = 0;

	void put(std::uint8_t c) {
		if (n < cap)
			p[n] = c;
		++n;
	}

	void put(const char* s) {
		while (*s) put(static_cast<std::uint8_t>(*s++));
	}
};

const char kAlnum[] = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ0123456789";

// JSON generator parameters (one struct per workload family).
struct JsonParams {
	double		  p_object, p_array;  // else scalar
	int			  fan_lo, fan_hi;
	int			  max_depth;
	int			  str_lo, str_hi;
	double		  p_escape_string;	   // fraction of strings that carry escapes
	double		  p_long_string;	   // chance a scalar is a long string
	int			  long_lo, long_hi;	   // long string length bounds
};

void ws(Rng& r, Out& o) {
	const int k = static_cast<int>(r.range(0, 2));
	for (int i = 0; i < k; ++i) o.put(r.chance(0.5) ? ' ' : '\n');
}

// One string body: printable ASCII (structural bytes included, so masking is
// exercised), occasional 2-byte UTF-8, and with probability `p_esc` escape
// sequences: \" or a run of 1-4 backslashes (odd runs end in an escaped quote or
// 'n', so the output stays valid JSON).
void string_body(Rng& r, Out& o, std::uint64_t len, bool escapes) {
	std::uint64_t i = 0;
	while (i < len) {
		if (escapes && r.chance(0.08)) {
			const int k = static_cast<int>(r.range(1, 4));
			if (r.chance(0.4)) {
				o.put("\\\"");
				i += 2;
				continue;
			}
			for (int j = 0; j < k; ++j) o.put('\\');
			if (k & 1)
				o.put(r.chance(0.5) ? '"' : 'n');
			i += static_cast<std::uint64_t>(k + (k & 1));
			continue;
		}
		const std::uint64_t u = r.range(0, 99);
		if (u < 2) {
			o.put(0xC3);
			o.put(static_cast<std::uint8_t>(0xA0 + r.range(0, 15)));
			i += 2;
		} else {
			std::uint8_t c = static_cast<std::uint8_t>(r.range(0x20, 0x7E));
			if (c == '"' || c == '\\')
				c = 'x';
			o.put(c);
			++i;
		}
	}
}

void json_string(Rng& r, Out& o, const JsonParams& P, bool long_ok) {
	o.put('"');
	if (long_ok && P.p_long_string > 0 && r.chance(P.p_long_string)) {
		string_body(r, o, r.range(P.long_lo, P.long_hi), true);
	} else {
		const bool esc = r.chance(P.p_escape_string);
		string_body(r, o, r.range(P.str_lo, P.str_hi), esc);
	}
	o.put('"');
}

void json_key(Rng& r, Out& o) {
	o.put('"');
	const int k = static_cast<int>(r.range(4, 12));
	for (int i = 0; i < k; ++i) o.put(static_cast<std::uint8_t>('a' + r.range(0, 25)));
	o.put('"');
}

void json_number(Rng& r, Out& o) {
	if (r.chance(0.3))
		o.put('-');
	const int nd = static_cast<int>(r.range(1, 9));
	o.put(static_cast<std::uint8_t>('1' + r.range(0, 8)));
	for (int i = 1; i < nd; ++i) o.put(static_cast<std::uint8_t>('0' + r.range(0, 9)));
	if (r.chance(0.4)) {
		o.put('.');
		const int nf = static_cast<int>(r.range(1, 6));
		for (int i = 0; i < nf; ++i) o.put(static_cast<std::uint8_t>('0' + r.range(0, 9)));
		if (r.chance(0.2)) {
			o.put('e');
			o.put(r.chance(0.5) ? '+' : '-');
			o.put(static_cast<std::uint8_t>('0' + r.range(0, 9)));
		}
	}
}

void json_scalar(Rng& r, Out& o, const JsonParams& P) {
	const std::uint64_t u = r.range(0, 9);
	if (u < 4)
		json_string(r, o, P, true);
	else if (u < 8)
		json_number(r, o);
	else if (u == 8)
		o.put(r.chance(0.5) ? "true" : "false");
	else
		o.put("null");
}

// Iterative DFS with an explicit stack, so depth 1024 needs no recursion.
struct Frame {
	bool object;
	int	 remaining;
	bool first;
};

std::uint64_t gen_json(std::uint64_t seed, std::uint64_t target, const JsonParams& P, Out& o) {
	Rng				   r(seed);
	std::vector<Frame> st;
	st.reserve(static_cast<std::size_t>(P.max_depth) + 2);
	o.put('[');
	st.push_back({false, -1, true});  // top level: unbounded array
	auto value_start = [&](int depth) {
		// depth: number of open containers including the top-level array
		const double u = r.unit();
		if (depth < P.max_depth && u < P.p_object) {
			o.put('{');
			st.push_back({true, static_cast<int>(r.range(P.fan_lo, P.fan_hi)), true});
		} else if (depth < P.max_depth && u < P.p_object + P.p_array) {
			o.put('[');
			st.push_back({false, static_cast<int>(r.range(P.fan_lo, P.fan_hi)), true});
		} else {
			json_scalar(r, o, P);
		}
	};
	while (!st.empty()) {
		Frame& f = st.back();
		const bool budget_hit = o.n >= target;
		if (f.remaining == 0 || (budget_hit && !(st.size() == 1 && f.first))) {
			ws(r, o);
			o.put(f.object ? '}' : ']');
			st.pop_back();
			continue;
		}
		if (f.remaining > 0)
			--f.remaining;
		if (!f.first)
			o.put(',');
		f.first = false;
		ws(r, o);
		if (f.object) {
			json_key(r, o);
			ws(r, o);
			o.put(':');
			ws(r, o);
		}
		value_start(static_cast<int>(st.size()));
	}
	return o.n;
}

// Deep-nesting stress: a top-level array of "spines".  Each spine draws its depth
// D uniformly from [1, 1024] and nests D containers; every level carries 0-2
// sibling scalars before and after the spine child, and a sibling is a long
// (1-64 KiB) escape-bearing string with probability P.p_long_string.
std::uint64_t gen_deep(std::uint64_t seed, std::uint64_t target, const JsonParams& P, Out& o) {
	Rng				  r(seed);
	std::vector<char> closers;
	std::vector<int>  after;
	bool			  first_top = true;
	o.put('[');
	auto sibling = [&](bool object, bool& first) {
		if (!first)
			o.put(',');
		first = false;
		ws(r, o);
		if (object) {
			json_key(r, o);
			o.put(':');
		}
		if (r.chance(P.p_long_string)) {
			o.put('"');
			string_body(r, o, r.range(P.long_lo, P.long_hi), true);
			o.put('"');
		} else {
			json_scalar(r, o, P);
		}
	};
	while (o.n < target) {
		if (!first_top)
			o.put(',');
		first_top	 = false;
		const int D	 = static_cast<int>(r.range(1, static_cast<std::uint64_t>(P.max_depth)));
		bool first	 = true;
		bool object	 = false;
		for (int lvl = 0; lvl < D && o.n < target; ++lvl) {
			// open this level's container as the spine child of the previous level
			if (lvl > 0) {
				if (!first)
					o.put(',');
				ws(r, o);
				if (object) {
					json_key(r, o);
					o.put(':');
				}
			}
			object = r.chance(0.5);
			o.put(object ? '{' : '[');
			closers.push_back(object ? '}' : ']');
			first = true;
			for (int k = static_cast<int>(r.range(0, 2)); k > 0; --k) sibling(object, first);
			after.push_back(static_cast<int>(r.range(0, 2)));
		}
		while (!closers.empty()) {
			const bool obj = closers.back() == '}';
			bool	   f   = false;
			for (int k = after.back(); k > 0 && o.n < target; --k) sibling(obj, f);
			o.put(closers.back());
			closers.pop_back();
			after.pop_back();
		}
	}
	o.put(']');
	return o.n;
}

}  // namespace

extern "C" {

// mode 0: single-document / batched-document JSON (tree 40% object, 30% array,
//         30% scalar; fanout U[1,8]; depth <= 16; strings 0-64 B, 5% with escapes).
// mode 1: deep-nesting stress (depth drawn up to 1024, ~20% of bytes in 1-64 KiB
//         strings with escape runs).
// Writes at most `cap` bytes to `out` and returns the full generated length (the
// document is complete only when the return value is <= cap).
std::uint64_t pars_synth_json(
	std::uint64_t seed, std::uint64_t target, int mode, std::uint8_t* out, std::uint64_t cap
) {
	Out o {out, cap};
	if (mode == 1) {
		const JsonParams P {0.0, 0.0, 1, 1, 1024, 0, 64, 0.05, 0.0008, 1024, 65536};
		return gen_deep(seed, target, P, o);
	}
	const JsonParams P {0.40, 0.30, 1, 8, 16, 0, 64, 0.05, 0.0, 0, 0};
	return gen_json(seed, target, P, o);
}

// 16 columns, LF records; unquoted fields U[0,24] alphanumerics; 10% quoted fields
// whose U[0,24] content positions are ',' / LF / '""' at 5% each.  Records are
// emitted until the size reaches `target` (whole records only).
std::uint64_t pars_synth_csv(std::uint64_t seed, std::uint64_t target, std::uint8_t* out,
							 std::uint64_t cap) {
	Rng r(seed);
	Out o {out, cap};
	while (o.n < target) {
		for (int col = 0; col < 16; ++col) {
			if (col)
				o.put(',');
			const std::uint64_t len = r.range(0, 24);
			if (r.chance(0.10)) {
				o.put('"');
				for (std::uint64_t i = 0; i < len; ++i) {
					const std::uint64_t u = r.range(0, 99);
					if (u < 5)
						o.put(',');
					else if (u < 10)
						o.put('\n');
					else if (u < 15)
						o.put("\"\"");
					else
						o.put(static_cast<std::uint8_t>(kAlnum[r.range(0, 61)]));
				}
				o.put('"');
			} else {
				for (std::uint64_t i = 0; i < len; ++i)
					o.put(static_cast<std::uint8_t>(kAlnum[r.range(0, 61)]));
			}
		}
		o.put('\n');
	}
	return o.n;
}

// Documents for the multi-descriptor grammars (kind 0 TOML, 1 C-like, 2 INI, 3 XML).
// Each mixes every lexical mode of its grammar with the grammar's structural bytes
// placed both outside and inside those modes (strings, comments), so the general
// kernel's state carries are exercised at every distance.  Whole records are emitted
// until the size reaches `target`.
std::uint64_t pars_synth_config(std::uint64_t seed, int kind, std::uint64_t target, std::uint8_t* out,
								std::uint64_t cap) {
	Rng r(seed);
	Out o {out, cap};
	auto word = [&](std::uint64_t lo, std::uint64_t hi) {
		const std::uint64_t len = r.range(lo, hi);
		for (std::uint64_t i = 0; i < len; ++i) o.put(static_cast<std::uint8_t>(kAlnum[r.range(0, 61)]));
	};
	// free text that may carry any of `noise` (structural outside the mode)
	auto text = [&](std::uint64_t lo, std::uint64_t hi, const char* noise, double p) {
		const std::uint64_t len	 = r.range(lo, hi);
		const std::uint64_t nlen = std::strlen(noise);
		for (std::uint64_t i = 0; i < len; ++i) {
			if (r.chance(p))
				o.put(static_cast<std::uint8_t>(noise[r.range(0, nlen - 1)]));
			else if (r.chance(0.15))
				o.put(' ');
			else
				o.put(static_cast<std::uint8_t>(kAlnum[r.range(0, 61)]));
		}
	};
	while (o.n < target) {
		const std::uint64_t u = r.range(0, 99);
		switch (kind) {
			case 0: {  // TOML
				if (u < 8) {
					const bool arr = r.chance(0.3);	 // [[array table]] or [table]
					o.put(arr ? "[[" : "[");
					word(3, 10);
					if (r.chance(0.5)) {
						o.put('.');
						word(2, 8);
					}
					o.put(arr ? "]]" : "]");
				} else if (u < 18) {
					o.put('#');
					text(0, 40, "{}[],=\"'.", 0.15);
				} else {
					word(2, 12);
					if (r.chance(0.2)) {
						o.put('.');
						word(2, 8);
					}
					o.put(" = ");
					const std::uint64_t v = r.range(0, 99);
					if (v < 30) {
						o.put('"');
						const std::uint64_t len = r.range(0, 40);
						for (std::uint64_t i = 0; i < len; ++i) {
							const std::uint64_t w = r.range(0, 99);
							if (w < 4)
								o.put("\\\"");
							else if (w < 7)
								o.put("\\\\");
							else if (w < 14)
								o.put(static_cast<std::uint8_t>("{}[],=#'."[r.range(0, 8)]));
							else
								o.put(static_cast<std::uint8_t>(kAlnum[r.range(0, 61)]));
						}
						o.put('"');
					} else if (v < 45) {
						o.put('\'');
						text(0, 30, "{}[],=#\"\\.", 0.15);
						o.put('\'');
					} else if (v < 60) {
						o.put('[');
						const std::uint64_t k = r.range(0, 6);
						for (std::uint64_t i = 0; i < k; ++i) {
							if (i)
								o.put(", ");
							word(1, 6);
						}
						o.put(']');
					} else if (v < 70) {
						o.put("{ ");
						word(1, 6);
						o.put(" = ");
						word(1, 6);
						o.put(", ");
						word(1, 6);
						o.put(" = \"");
						text(0, 12, "{},", 0.2);
						o.put("\" }");
					} else {
						word(1, 10);
					}
					if (r.chance(0.1)) {
						o.put(" # ");
						text(0, 20, "{}[],=\"'", 0.2);
					}
				}
				o.put('\n');
				break;
			}
			case 1: {  // C-like
				if (u < 15) {
					o.put("/*");
					text(0, 60, "{};/\n", 0.1);
					if (r.chance(0.3))
						o.put("**");
					o.put("*/");
				} else if (u < 30) {
					o.put("//");
					text(0, 50, "{};/*", 0.12);
					o.put('\n');
				} else if (u < 45) {
					o.put(r.chance(0.5) ? "{\n" : "}\n");
				} else {
					word(1, 10);
					o.put(' ');
					word(1, 10);
					o.put(r.chance(0.7) ? ";\n" : "; ");
				}
				break;
			}
			case 2: {  // INI
				if (u < 10) {
					o.put('[');
					word(3, 12);
					o.put("]\n");
				} else if (u < 25) {
					o.put(';');
					text(0, 50, "[]=#", 0.15);
					o.put('\n');
				} else if (u < 30) {
					o.put('\n');
				} else {
					word(1, 12);
					o.put(r.chance(0.5) ? " = " : "=");
					word(0, 20);
					o.put('\n');
				}
				break;
			}
			default: {	// XML
				if (u < 10) {
					o.put("<?");
					word(3, 6);
					o.put(" v=\"1.0\"?>");
				} else if (u < 20) {
					o.put("<!");
					word(3, 8);
					o.put(' ');
					word(1, 10);
					o.put('>');
				} else if (u < 55) {
					o.put('<');
					word(1, 8);
					const std::uint64_t na = r.range(0, 3);
					for (std::uint64_t i = 0; i < na; ++i) {
						o.put(' ');
						word(1, 6);
						o.put('=');
						if (r.chance(0.6)) {
							o.put('"');
							text(0, 20, "<>/='", 0.15);
							o.put('"');
						} else {
							o.put('\'');
							text(0, 20, "<>/=\"", 0.15);
							o.put('\'');
						}
					}
					o.put(r.chance(0.2) ? "/>" : ">");
				} else if (u < 75) {
					o.put("</");
					word(1, 8);
					o.put('>');
				} else {
					text(1, 60, ">/='\"&;", 0.08);
				}
				if (r.chance(0.3))
					o.put('\n');
				break;
			}
		}
	}
	return o.n;
}

// n bytes drawn uniformly from `alphabet[0..alen)`.
void pars_synth_alpha(std::uint64_t seed, const std::uint8_t* alphabet, std::uint64_t alen,
					  std::uint8_t* out, std::uint64_t n) {
	Rng r(seed);
	for (std::uint64_t i = 0; i < n; ++i) out[i] = alphabet[r.next() % alen];
}

// Log-normal document sizes (median `median`, shape `sigma`) clamped to [lo, hi].
void pars_synth_lognormal_sizes(std::uint64_t seed, std::uint64_t count, double median,
								double sigma, std::uint64_t lo, std::uint64_t hi,
								std::uint64_t* out) {
	Rng r(seed);
	for (std::uint64_t i = 0; i < count; ++i) {
		// Box-Muller
		double u1 = r.unit(), u2 = r.unit();
		if (u1 < 1e-300)
			u1 = 1e-300;
		const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
		double		 v = median * std::exp(sigma * z);
		if (v < static_cast<double>(lo))
			v = static_cast<double>(lo);
		if (v > static_cast<double>(hi))
			v = static_cast<double>(hi);
		out[i] = static_cast<std::uint64_t>(v);
	}
}

}  // extern "C"
