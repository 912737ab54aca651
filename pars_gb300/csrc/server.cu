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
// Results come back through the worker's pinned staging.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pars_gb300.h"

namespace {

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
	std::vector<std::uint32_t> structural;
	std::vector<std::int32_t>  pair_pos;
	std::int32_t		   balanced = 1, well_formed = 1, max_depth = 0, unclosed = 0;
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
	std::string						  err;
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
		auto& q = *batch[0];
		if (grow_pinned(w, r.n_struct * (pairs ? 2 : 1)))
			return fail_all(PARS_ENOMEM);
		if (r.n_struct)
			cudaMemcpyAsync(w.h_u32, r.structural, r.n_struct * 4, cudaMemcpyDeviceToHost, w.stream);
		if (pairs && r.pair_pos && r.n_struct)
			cudaMemcpyAsync(w.h_u32 + r.n_struct, r.pair_pos, r.n_struct * 4, cudaMemcpyDeviceToHost, w.stream);
		if (cudaStreamSynchronize(w.stream) != cudaSuccess) {
			cudaGetLastError();
			return fail_all(PARS_ECUDA);
		}
		q.structural.assign(w.h_u32, w.h_u32 + r.n_struct);
		if (pairs && r.pair_pos)
			q.pair_pos.assign(reinterpret_cast<const std::int32_t*>(w.h_u32) + r.n_struct,
							  reinterpret_cast<const std::int32_t*>(w.h_u32) + 2 * r.n_struct);
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
	// every request's offsets (and pairs) back to back through the pinned staging
	std::size_t words = 0;
	for (std::uint32_t i = 0; i < nd; ++i) words += static_cast<std::size_t>(rec[nd + i]) * (pairs ? 2 : 1);
	if (grow_pinned(w, words))
		return fail_all(PARS_ENOMEM);
	std::size_t at = 0;
	for (std::uint32_t i = 0; i < nd; ++i) {
		const std::uint32_t so = rec[i], ns = rec[nd + i];
		if (ns) {
			cudaMemcpyAsync(w.h_u32 + at, br.structural + so, ns * 4ull, cudaMemcpyDeviceToHost, w.stream);
			if (pairs && br.pair_pos)
				cudaMemcpyAsync(w.h_u32 + at + ns, br.pair_pos + so, ns * 4ull, cudaMemcpyDeviceToHost, w.stream);
		}
		at += static_cast<std::size_t>(ns) * (pairs ? 2 : 1);
	}
	if (cudaStreamSynchronize(w.stream) != cudaSuccess) {
		cudaGetLastError();
		return fail_all(PARS_ECUDA);
	}
	at = 0;
	for (std::uint32_t i = 0; i < nd; ++i) {
		auto&				q  = *batch[i];
		const std::uint32_t ns = rec[nd + i];
		q.structural.assign(w.h_u32 + at, w.h_u32 + at + ns);
		if (pairs && br.pair_pos)
			q.pair_pos.assign(reinterpret_cast<const std::int32_t*>(w.h_u32) + at + ns,
							  reinterpret_cast<const std::int32_t*>(w.h_u32) + at + 2 * ns);
		at += static_cast<std::size_t>(ns) * (pairs ? 2 : 1);
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
			s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty(); });
			if (s->stop)
				return;
			// admission: the oldest request's plan, then every pending request of that
			// plan that fits the free room of this worker's arena slice
			const int	  plan	= s->pending.front()->plan;
			std::uint64_t room	= w->cap;
			const std::uint32_t maxd = s->cfg.max_batch_docs ? s->cfg.max_batch_docs : 1;
			for (auto it = s->pending.begin(); it != s->pending.end() && batch.size() < maxd;) {
				auto& r = *it;
				if (r->plan == plan && (r->n <= room || batch.empty())) {
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
		}
		s->cv_done.notify_all();
	}
}

void fill(const Request& r, pars_server_result* out) {
	std::memset(out, 0, sizeof *out);
	out->status		   = r.status;
	out->structural	   = r.structural.data();
	out->pair_pos	   = r.pair_pos.empty() ? nullptr : r.pair_pos.data();
	out->n_struct	   = r.structural.size();
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
	delete s;
	return 0;
}

int pars_server_plan_load(pars_server* s, const void* plan, size_t len, int* plan_id) {
	if (!s || !plan || !plan_id)
		return PARS_EINVAL;
	std::lock_guard<std::mutex> lk(s->mu);
	for (auto& w : s->workers) {
		int id = -1;
		if (int rc = pars_plan_load(w->ctx, plan, len, &id))
			return rc;
		w->plan_ids.push_back(id);
	}
	s->plans.emplace_back(static_cast<const std::uint8_t*>(plan), static_cast<const std::uint8_t*>(plan) + len);
	*plan_id = static_cast<int>(s->plans.size()) - 1;
	return 0;
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
	s->all.erase(it);
	return 0;
}

}  // extern "C"
