// server.cu — continuous-batching request server over the C ABI (host code).
//
// Requests (a document and a plan) are submitted from any thread and queued.  Each
// of the server's workers owns a context, a stream, a slice of the device input
// arena and pinned host staging.  A worker takes the oldest pending request's plan,
// admits every pending request of that plan that fits the free room of its arena
// slice (up to max_batch_docs), uploads them back to back, scans them in ONE
// pars_scan_batch launch and copies each request's results into host memory.
// While one worker's launch runs on the GPU, another is already admitting and
// uploading the requests that arrived meanwhile: their work overlaps on the device.
// A launch of a single request (always, with max_batch_docs = 1: the plain
// per-request path the batched path is measured against) is one pars_scan_device.
// Results land in a server-wide pool of pinned host memory: each request's offsets
// (and pairs) are copied from the device straight into its own slice, which the
// client reads in place until it releases the request.  A result the pool cannot
// hold goes through the worker's pinned staging into the request's own buffers.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pars_gb300.h"

namespace {

// Requests from this size up run alone (the single-document launch).
constexpr std::uint64_t kServeSoloBytes = 1ull << 20;

std::uint64_t now_ns() {
	return static_cast<std::uint64_t>(std::chrono::duration_cast<std::chrono::nanoseconds>(
										  std::chrono::steady_clock::now().time_since_epoch())
										  .count());
}

struct Request {
	std::uint64_t		   ticket = 0;
	int					   plan	  = 0;	// server plan id
	const std::uint8_t*	   data	  = nullptr;
	std::uint64_t		   n	  = 0;
	std::uint32_t		   flags  = 0;
	std::uint64_t		   submit_ns = 0, start_ns = 0, done_ns = 0;
	std::uint32_t		   batch_docs = 0;
	int					   status = PARS_EAGAIN;
	std::vector<std::uint32_t> structural;	 // when the result is not in the pool
	std::vector<std::int32_t>  pair_pos;
	std::uint32_t*		   pooled = nullptr;  // in the pool: offsets, then pairs
	std::size_t			   pooled_bytes = 0;
	std::uint64_t		   n_struct = 0;
	bool				   has_pairs = false;
	std::int32_t		   balanced = 1, well_formed = 1, max_depth = 0, unclosed = 0;
};

// Pinned host memory for results: first fit over a free list of (offset, size),
// neighbours merged on release.  Thread-safe.
class ResultPool {
  public:
	int init(std::size_t bytes) {
		if (cudaHostAlloc(reinterpret_cast<void**>(&base_), bytes, cudaHostAllocDefault) != cudaSuccess) {
			cudaGetLastError();
			base_ = nullptr;
			return PARS_ENOMEM;
		}
		cap_ = bytes;
		free_.emplace(0, bytes);
		return 0;
	}
	void destroy() {
		if (base_)
			cudaFreeHost(base_);
		base_ = nullptr;
	}
	void* alloc(std::size_t bytes) {
		bytes = (bytes + 255) & ~std::size_t(255);
		std::lock_guard<std::mutex> lk(mu_);
		for (auto it = free_.begin(); it != free_.end(); ++it) {
			if (it->second < bytes)
				continue;
			const std::size_t off = it->first, left = it->second - bytes;
			free_.erase(it);
			if (left)
				free_.emplace(off + bytes, left);
			return base_ + off;
		}
		return nullptr;
	}
	void release(void* p, std::size_t bytes) {
		if (!p)
			return;
		bytes = (bytes + 255) & ~std::size_t(255);
		std::lock_guard<std::mutex> lk(mu_);
		std::size_t off = static_cast<std::uint8_t*>(p) - base_;
		auto		nx	= free_.lower_bound(off);
		if (nx != free_.end() && off + bytes == nx->first) {  // merge with the next block
			bytes += nx->second;
			nx = free_.erase(nx);
		}
		if (nx != free_.begin()) {	// merge with the previous block
			auto pv = std::prev(nx);
			if (pv->first + pv->second == off) {
				pv->second += bytes;
				return;
			}
		}
		free_.emplace(off, bytes);
	}

  private:
	std::mutex						   mu_;
	std::uint8_t*					   base_ = nullptr;
	std::size_t						   cap_	 = 0;
	std::map<std::size_t, std::size_t> free_;
};

struct Worker {
	pars_ctx*			   ctx	  = nullptr;
	cudaStream_t		   stream = nullptr;
	std::uint8_t*		   d_in	  = nullptr;  // this worker's slice of the input arena
	std::uint64_t		   cap	  = 0;
	std::vector<int>	   plan_ids;		  // server plan id -> this context's plan id
	std::thread			   thread;
	// pinned staging for per-document results
	std::uint32_t*		   h_u32  = nullptr;
	std::size_t			   h_cap  = 0;
};

}  // namespace

struct pars_server {
	pars_server_config				  cfg {};
	std::vector<std::unique_ptr<Worker>> workers;
	std::vector<std::vector<std::uint8_t>> plans;
	std::mutex						  mu;
	std::condition_variable			  cv_work, cv_done;
	std::deque<std::shared_ptr<Request>> pending;
	std::unordered_map<std::uint64_t, std::shared_ptr<Request>> all;
	std::uint64_t					  next_ticket = 1;
	bool							  stop		  = false;
	// plan loads touch every worker's context: they wait until no launch is in
	// flight (busy) and hold admissions back meanwhile (loading)
	int								  busy		  = 0;
	int								  loading	  = 0;
	std::string						  err;
	ResultPool						  pool;
};

namespace {

int grow_pinned(Worker& w, std::size_t words) {
	if (words <= w.h_cap)
		return 0;
	if (w.h_u32)
		cudaFreeHost(w.h_u32);
	w.h_u32 = nullptr;
	w.h_cap = 0;
	const std::size_t want = words + words / 2 + 1024;
	if (cudaHostAlloc(reinterpret_cast<void**>(&w.h_u32), want * 4, cudaHostAllocDefault) != cudaSuccess) {
		cudaGetLastError();
		return PARS_ENOMEM;
	}
	w.h_cap = want;
	return 0;
}

// A pool slice of `words` 32-bit words for request q's results, or null when the
// pool cannot hold them (the caller stages them instead).
std::uint32_t* take_pooled(pars_server* s, Request& q, std::size_t words) {
	if (words == 0)
		return nullptr;
	void* p = s->pool.alloc(words * 4);
	if (p) {
		q.pooled	   = static_cast<std::uint32_t*>(p);
		q.pooled_bytes = words * 4;
	}
	return static_cast<std::uint32_t*>(p);
}

// Runs one launch over `batch` (all of one plan) on worker `w`; fills the requests.
void run_batch(pars_server* s, Worker& w, std::vector<std::shared_ptr<Request>>& batch) {
	const int			plan = w.plan_ids[batch[0]->plan];
	const std::uint32_t nd	 = static_cast<std::uint32_t>(batch.size());
	std::vector<std::uint64_t> offs(nd + 1, 0);
	for (std::uint32_t i = 0; i < nd; ++i) offs[i + 1] = offs[i] + batch[i]->n;
	auto fail_all = [&](int code) {
		for (auto& r : batch) r->status = code;
	};
	for (std::uint32_t i = 0; i < nd; ++i)
		if (batch[i]->n)
			if (cudaMemcpyAsync(w.d_in + offs[i], batch[i]->data, batch[i]->n, cudaMemcpyHostToDevice, w.stream)
				!= cudaSuccess) {
				cudaGetLastError();
				return fail_all(PARS_ECUDA);
			}
	const std::uint32_t flags = batch[0]->flags | PARS_RUN_PAIRS;
	const bool			pairs = (flags & PARS_WANT_PAIRS) != 0;
	if (nd == 1) {
		// one request (the plain path, or a lone request): one single-document launch
		pars_device_result r {};
		const int rc = pars_scan_device(w.ctx, plan, w.d_in, batch[0]->n, flags, w.stream, &r);
		if (rc)
			return fail_all(rc);
		auto&			  q		= *batch[0];
		const bool		  wantp = pairs && r.pair_pos;
		const std::size_t words = r.n_struct * (wantp ? 2 : 1);
		q.n_struct				= r.n_struct;
		q.has_pairs				= wantp;
		std::uint32_t* dst		= take_pooled(s, q, words);
		if (!dst) {
			if (grow_pinned(w, words))
				return fail_all(PARS_ENOMEM);
			dst = w.h_u32;
		}
		if (r.n_struct)
			cudaMemcpyAsync(dst, r.structural, r.n_struct * 4, cudaMemcpyDeviceToHost, w.stream);
		if (wantp && r.n_struct)
			cudaMemcpyAsync(dst + r.n_struct, r.pair_pos, r.n_struct * 4, cudaMemcpyDeviceToHost, w.stream);
		if (cudaStreamSynchronize(w.stream) != cudaSuccess) {
			cudaGetLastError();
			return fail_all(PARS_ECUDA);
		}
		if (!q.pooled) {
			q.structural.assign(dst, dst + r.n_struct);
			if (wantp)
				q.pair_pos.assign(reinterpret_cast<const std::int32_t*>(dst) + r.n_struct,
								  reinterpret_cast<const std::int32_t*>(dst) + 2 * r.n_struct);
		}
		q.balanced	  = r.balanced;
		q.well_formed = r.well_formed;
		q.max_depth	  = r.max_depth;
		q.unclosed	  = r.unclosed_mode;
		q.status	  = 0;
		return;
	}
	pars_batch_result br {};
	const int rc = pars_scan_batch(w.ctx, plan, w.d_in, offs.data(), nd, flags, w.stream, &br);
	if (rc)
		return fail_all(rc);
	// per-document records (8 arrays of nd words) through pinned staging
	if (grow_pinned(w, static_cast<std::size_t>(nd) * 8))
		return fail_all(PARS_ENOMEM);
	const void* recs[8] = {br.struct_off, br.n_struct, br.unclosed_mode, br.balanced,
						   br.well_formed, br.max_depth, nullptr, nullptr};
	for (int k = 0; k < 6; ++k)
		if (recs[k])
			cudaMemcpyAsync(w.h_u32 + static_cast<std::size_t>(k) * nd, recs[k], nd * 4, cudaMemcpyDeviceToHost,
							w.stream);
	if (cudaStreamSynchronize(w.stream) != cudaSuccess) {
		cudaGetLastError();
		return fail_all(PARS_ECUDA);
	}
	std::vector<std::uint32_t> rec(w.h_u32, w.h_u32 + static_cast<std::size_t>(nd) * 6);
	// every request's offsets (and pairs) into its pool slice, or back to back
	// through the pinned staging when the pool cannot hold it
	const bool				   wantp = pairs && br.pair_pos;
	std::vector<std::uint32_t*> dst(nd, nullptr);
	std::size_t				   words = 0;
	for (std::uint32_t i = 0; i < nd; ++i) {
		auto&			  q	 = *batch[i];
		const std::size_t ws = static_cast<std::size_t>(rec[nd + i]) * (wantp ? 2 : 1);
		q.n_struct			 = rec[nd + i];
		q.has_pairs			 = wantp;
		dst[i]				 = take_pooled(s, q, ws);
		if (!dst[i])
			words += ws;
	}
	if (grow_pinned(w, words))
		return fail_all(PARS_ENOMEM);
	std::size_t at = 0;
	for (std::uint32_t i = 0; i < nd; ++i) {
		const std::uint32_t so = rec[i], ns = rec[nd + i];
		if (!dst[i]) {
			dst[i] = w.h_u32 + at;
			at += static_cast<std::size_t>(ns) * (wantp ? 2 : 1);
		}
		if (ns) {
			cudaMemcpyAsync(dst[i], br.structural + so, ns * 4ull, cudaMemcpyDeviceToHost, w.stream);
			if (wantp)
				cudaMemcpyAsync(dst[i] + ns, br.pair_pos + so, ns * 4ull, cudaMemcpyDeviceToHost, w.stream);
		}
	}
	if (cudaStreamSynchronize(w.stream) != cudaSuccess) {
		cudaGetLastError();
		return fail_all(PARS_ECUDA);
	}
	for (std::uint32_t i = 0; i < nd; ++i) {
		auto&				q  = *batch[i];
		const std::uint32_t ns = rec[nd + i];
		if (!q.pooled) {
			q.structural.assign(dst[i], dst[i] + ns);
			if (wantp)
				q.pair_pos.assign(reinterpret_cast<const std::int32_t*>(dst[i]) + ns,
								  reinterpret_cast<const std::int32_t*>(dst[i]) + 2 * ns);
		}
		q.unclosed	  = static_cast<std::int32_t>(rec[2 * nd + i]);
		q.balanced	  = br.balanced ? static_cast<std::int32_t>(rec[3 * nd + i]) : 1;
		q.well_formed = br.well_formed ? static_cast<std::int32_t>(rec[4 * nd + i]) : 1;
		q.max_depth	  = br.max_depth ? static_cast<std::int32_t>(rec[5 * nd + i]) : 0;
	}
	for (auto& r : batch) r->status = 0;
}

void worker_loop(pars_server* s, Worker* w) {
	cudaSetDevice(s->cfg.device);
	for (;;) {
		std::vector<std::shared_ptr<Request>> batch;
		{
			std::unique_lock<std::mutex> lk(s->mu);
			s->cv_work.wait(lk, [&] { return s->stop || (!s->pending.empty() && !s->loading); });
			if (s->stop)
				return;
			// admission: the oldest request's plan, then every pending request of that
			// plan that fits the free room of this worker's arena slice.  A large
			// request runs alone on the whole grid (in a batch launch a document
			// stays on one CTA, and every request of the batch would wait for it);
			// large requests are never folded into a batch of small ones.
			const int	  plan	= s->pending.front()->plan;
			std::uint64_t room	= w->cap;
			const bool	  solo	= s->pending.front()->n >= kServeSoloBytes;
			const std::uint32_t maxd = solo ? 1u : (s->cfg.max_batch_docs ? s->cfg.max_batch_docs : 1);
			for (auto it = s->pending.begin(); it != s->pending.end() && batch.size() < maxd;) {
				auto& r = *it;
				if (r->plan == plan && (r->n <= room || batch.empty()) && (batch.empty() || r->n < kServeSoloBytes)) {
					if (r->n > w->cap) {
						// never fits: fail it rather than block the queue
						r->status  = PARS_ERANGE;
						r->done_ns = now_ns();
						it		   = s->pending.erase(it);
						s->cv_done.notify_all();
						continue;
					}
					room -= r->n;
					batch.push_back(r);
					it = s->pending.erase(it);
				} else {
					++it;
				}
			}
			if (!batch.empty())
				++s->busy;
		}
		if (batch.empty())
			continue;
		const std::uint64_t t0 = now_ns();
		for (auto& r : batch) {
			r->start_ns	  = t0;
			r->batch_docs = static_cast<std::uint32_t>(batch.size());
		}
		run_batch(s, *w, batch);
		const std::uint64_t t1 = now_ns();
		{
			std::lock_guard<std::mutex> lk(s->mu);
			for (auto& r : batch) r->done_ns = t1;
			--s->busy;
		}
		s->cv_done.notify_all();
	}
}

void fill(const Request& r, pars_server_result* out) {
	std::memset(out, 0, sizeof *out);
	out->status = r.status;
	if (r.pooled) {
		out->structural = r.pooled;
		out->pair_pos	= r.has_pairs ? reinterpret_cast<const std::int32_t*>(r.pooled) + r.n_struct : nullptr;
	} else {
		out->structural = r.structural.data();
		out->pair_pos	= r.pair_pos.empty() ? nullptr : r.pair_pos.data();
	}
	out->n_struct = r.status == 0 ? r.n_struct : 0;
	out->balanced	   = r.balanced;
	out->well_formed   = r.well_formed;
	out->max_depth	   = r.max_depth;
	out->unclosed_mode = r.unclosed;
	out->submit_ns	   = r.submit_ns;
	out->start_ns	   = r.start_ns;
	out->done_ns	   = r.done_ns;
	out->batch_docs	   = r.batch_docs;
}

}  // namespace

extern "C" {

int pars_server_create(const pars_server_config* cfg, pars_server** out) {
	if (!cfg || !out || cfg->arena_bytes == 0)
		return PARS_EINVAL;
	*out			 = nullptr;
	auto* s			 = new pars_server();
	s->cfg			 = *cfg;
	const int nw	 = cfg->workers ? static_cast<int>(cfg->workers) : 2;
	const std::uint64_t slice = (cfg->arena_bytes / static_cast<std::uint64_t>(nw)) & ~std::uint64_t(255);
	cudaSetDevice(cfg->device);
	for (int i = 0; i < nw; ++i) {
		auto w = std::make_unique<Worker>();
		if (int rc = pars_create(cfg->device, 0, &w->ctx)) {
			pars_server_destroy(s);
			return rc;
		}
		if (cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) != cudaSuccess
			|| cudaMalloc(reinterpret_cast<void**>(&w->d_in), slice + 256) != cudaSuccess) {
			cudaGetLastError();
			s->workers.push_back(std::move(w));
			pars_server_destroy(s);
			return PARS_ENOMEM;
		}
		w->cap = slice;
		s->workers.push_back(std::move(w));
	}
	// results in pinned memory; without it every result is staged and copied
	s->pool.init(static_cast<std::size_t>(cfg->result_mib ? cfg->result_mib : 1024u) << 20);
	for (auto& w : s->workers) w->thread = std::thread(worker_loop, s, w.get());
	*out = s;
	return 0;
}

int pars_server_destroy(pars_server* s) {
	if (!s)
		return PARS_EINVAL;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->stop = true;
	}
	s->cv_work.notify_all();
	for (auto& w : s->workers)
		if (w->thread.joinable())
			w->thread.join();
	cudaSetDevice(s->cfg.device);
	for (auto& w : s->workers) {
		if (w->stream)
			cudaStreamSynchronize(w->stream);
		if (w->d_in)
			cudaFree(w->d_in);
		if (w->h_u32)
			cudaFreeHost(w->h_u32);
		if (w->stream)
			cudaStreamDestroy(w->stream);
		if (w->ctx)
			pars_destroy(w->ctx);
	}
	s->pool.destroy();
	delete s;
	return 0;
}

int pars_server_plan_load(pars_server* s, const void* plan, size_t len, int* plan_id) {
	if (!s || !plan || !plan_id)
		return PARS_EINVAL;
	std::unique_lock<std::mutex> lk(s->mu);
	// a context belongs to one thread at a time: load into the workers' contexts only
	// while none of them runs a launch, and admit nothing until the load is done
	++s->loading;
	s->cv_done.wait(lk, [&] { return s->busy == 0; });
	int rc = 0;
	for (auto& w : s->workers) {
		int id = -1;
		if ((rc = pars_plan_load(w->ctx, plan, len, &id)) != 0)
			break;
		w->plan_ids.push_back(id);
	}
	if (rc == 0) {
		s->plans.emplace_back(static_cast<const std::uint8_t*>(plan), static_cast<const std::uint8_t*>(plan) + len);
		*plan_id = static_cast<int>(s->plans.size()) - 1;
	} else {
		// every worker's table stays as long as the server's
		for (auto& w : s->workers) w->plan_ids.resize(s->plans.size());
	}
	--s->loading;
	lk.unlock();
	s->cv_work.notify_all();
	return rc;
}

int pars_server_submit(pars_server* s, int plan_id, const uint8_t* data, uint64_t n, uint32_t flags,
					   uint64_t* ticket) {
	if (!s || !ticket || (n && !data))
		return PARS_EINVAL;
	if (n >= (1ull << 32))
		return PARS_ERANGE;
	auto r		 = std::make_shared<Request>();
	r->plan		 = plan_id;
	r->data		 = data;
	r->n		 = n;
	r->flags	 = flags & (PARS_WANT_PAIRS | PARS_RUN_PAIRS);
	r->submit_ns = now_ns();
	{
		std::lock_guard<std::mutex> lk(s->mu);
		if (plan_id < 0 || plan_id >= static_cast<int>(s->plans.size()))
			return PARS_EINVAL;
		r->ticket = s->next_ticket++;
		s->all.emplace(r->ticket, r);
		s->pending.push_back(r);
		*ticket = r->ticket;
	}
	s->cv_work.notify_one();
	return 0;
}

int pars_server_poll(pars_server* s, uint64_t ticket, pars_server_result* out) {
	if (!s || !out)
		return PARS_EINVAL;
	std::lock_guard<std::mutex> lk(s->mu);
	auto it = s->all.find(ticket);
	if (it == s->all.end())
		return PARS_EINVAL;
	if (it->second->done_ns == 0)
		return PARS_EAGAIN;
	fill(*it->second, out);
	return 0;
}

int pars_server_wait(pars_server* s, uint64_t ticket, pars_server_result* out) {
	if (!s || !out)
		return PARS_EINVAL;
	std::unique_lock<std::mutex> lk(s->mu);
	auto it = s->all.find(ticket);
	if (it == s->all.end())
		return PARS_EINVAL;
	auto r = it->second;
	s->cv_done.wait(lk, [&] { return r->done_ns != 0; });
	fill(*r, out);
	return 0;
}

int pars_server_release(pars_server* s, uint64_t ticket) {
	if (!s)
		return PARS_EINVAL;
	std::lock_guard<std::mutex> lk(s->mu);
	auto it = s->all.find(ticket);
	if (it == s->all.end() || it->second->done_ns == 0)
		return PARS_EINVAL;
	s->pool.release(it->second->pooled, it->second->pooled_bytes);
	it->second->pooled = nullptr;
	s->all.erase(it);
	return 0;
}

}  // extern "C"
