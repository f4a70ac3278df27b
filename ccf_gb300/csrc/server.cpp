/******************************************************************************
server.cpp -- device-memory estimate, asynchronous batches and the request
loop of include/ccf_gb300.h.

The reference runs one field per process and resets the device at every run
(include/ccf.cuh:151), so none of this has a counterpart there.  Each request
of the server gets its own handle: its own field, engine and CUDA stream, so
the kernels of concurrent requests overlap on the GPU.  Admission is FIFO
under two limits: a free slot (a worker thread) and the device bytes the
admitted requests hold, counted from admission until the caller releases the
request.
******************************************************************************/
#include "../../include/ccf_gb300.h"
#include "common.cuh"
#include "params.h"

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace
{

/* Upper estimate of the device bytes of one run (engine.cu's buffers). */
unsigned long long estimate_bytes(const ccf_params& p, const ccf::Derived& d)
{
	const unsigned long long N = (unsigned long long)d.num_stars;
	const unsigned long long R = (unsigned long long)d.num_roots;
	const unsigned long long nb = (unsigned long long)p.num_branches;
	const unsigned long long cols = (unsigned long long)(p.num_phi / p.num_branches + 1);
	const unsigned long long P1 = (unsigned long long)ccf::MAX_ORDER + 1;
	/* stars: generation and tree order, scratch copies, masses, split forms */
	unsigned long long b = N * (16 + 16 + 16 + 8 + 8 + 16 + 8);
	/* tree and FMM: at most ~N leaves; nodes <= 4/3 of the leaves, per node the
	   structure arrays and the multipole and local coefficients */
	const unsigned long long nodes = 2 * N + 64;
	b += nodes * (224 + 2 * P1 * 16);
	/* leaves: near lists (FP64 and double-float), local blocks, FP32 copy */
	b += nodes * (32 * 32 + 3 * P1 * 16 + P1 * 8 + 32 * 24 + 2 * P1 * 16 + 64);
	/* solver rows: centres and (branch, side) rows, 69 bytes per root */
	b += 3 * nb * R * 69;
	/* tracker: column tables (2 R slots of 8 bytes per phi step of every row),
	   solo-root lists (9 bytes per root of a row), row records and statistics */
	if (p.continuation == CCF_CONTINUATION_TRACK) b += 2 * nb * (cols / 2) * 2 * R * 8 + 2 * nb * R * 9 + 2 * nb * (40 + 40);
	/* outputs in the file layout (none on the device with host_outputs) */
	const unsigned long long pts = R * nb * cols;
	if (!p.host_outputs)
	{
		b += pts * (16 + 8);
		if (p.write_caustics) b += pts * 16;
		if (p.write_mu_length_scales) b += pts * 8;
	}
	return b + (64ull << 20);
}

bool derive(const ccf_params& p, ccf::Derived& d, std::string& msg)
{
	std::unique_ptr<ccf::StarField> sf;
	if (p.starfile[0])
	{
		sf.reset(new ccf::StarField());
		if (!ccf::read_star_file(p.starfile, *sf, msg)) return false;
	}
	return ccf::derive_params(p, sf.get(), d, msg);
}

double now_seconds(std::chrono::steady_clock::time_point t0)
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

} /* namespace */

/* ---------------- asynchronous batches ---------------- */

struct ccf_batch
{
	std::thread worker;
	std::mutex mu;
	std::condition_variable cv;
	bool done = false;
	ccf_status status = CCF_OK;
};

/* ---------------- serving ---------------- */

struct ServerRequest
{
	long long id = 0;
	ccf_params params;
	unsigned long long bytes = 0;
	ccf_handle* handle = nullptr;
	int state = CCF_REQUEST_QUEUED;
	ccf_status status = CCF_OK;
	bool deferred = false;
	bool counted = false;   /* its bytes are in bytes_in_use */
	double t_submit = 0, t_start = 0, t_end = 0;
};

struct ccf_server
{
	ccf_server_config cfg;
	std::chrono::steady_clock::time_point t0;
	std::mutex mu;
	std::condition_variable cv_work;   /* queue, budget or stop changed */
	std::condition_variable cv_done;   /* a request finished */
	std::deque<long long> queue;
	std::map<long long, std::unique_ptr<ServerRequest>> reqs;
	unsigned long long bytes_in_use = 0;
	long long next_id = 1;
	long long submitted = 0, admitted = 0, completed = 0, failed = 0, rejected = 0, deferred = 0;
	int running = 0;
	bool stop = false;
	std::vector<std::thread> workers;
};

static void server_worker(ccf_server* s)
{
	std::unique_lock<std::mutex> lk(s->mu);
	while (true)
	{
		ServerRequest* r = nullptr;
		while (!s->stop)
		{
			if (!s->queue.empty())
			{
				ServerRequest* head = s->reqs[s->queue.front()].get();
				if (head->bytes > s->cfg.hbm_budget)
				{
					/* can never fit: reject it */
					s->queue.pop_front();
					head->state = CCF_REQUEST_REJECTED;
					head->status = CCF_ERR_BUDGET;
					head->t_end = now_seconds(s->t0);
					s->rejected++;
					s->cv_done.notify_all();
					continue;
				}
				if (s->bytes_in_use + head->bytes <= s->cfg.hbm_budget)
				{
					s->queue.pop_front();
					r = head;
					break;
				}
				/* a slot is free but the memory is not: wait for a release */
				if (!head->deferred)
				{
					head->deferred = true;
					s->deferred++;
				}
			}
			s->cv_work.wait(lk);
		}
		if (!r) return;
		r->state = CCF_REQUEST_RUNNING;
		r->counted = true;
		s->bytes_in_use += r->bytes;
		s->admitted++;
		s->running++;
		r->t_start = now_seconds(s->t0);
		ccf_params p = r->params;
		const int verbose = s->cfg.verbose;
		lk.unlock();

		ccf_handle* h = nullptr;
		ccf_status st = ccf_create(&h);
		if (st == CCF_OK)
		{
			p.device = s->cfg.device;
			st = ccf_set_params(h, &p);
			if (st == CCF_OK) st = ccf_run(h, verbose);
		}

		lk.lock();
		r->handle = h;
		r->status = st;
		r->state = st == CCF_OK ? CCF_REQUEST_DONE : CCF_REQUEST_FAILED;
		r->t_end = now_seconds(s->t0);
		s->running--;
		if (st == CCF_OK) s->completed++;
		else s->failed++;
		s->cv_done.notify_all();
	}
}

extern "C" {

ccf_status ccf_estimate_device_bytes(const ccf_params* p, unsigned long long* bytes)
{
	if (!p || !bytes) return CCF_ERR_INVALID_ARGUMENT;
	ccf::Derived d;
	std::string msg;
	if (!derive(*p, d, msg)) return p->starfile[0] ? CCF_ERR_IO : CCF_ERR_INVALID_ARGUMENT;
	*bytes = estimate_bytes(*p, d);
	return CCF_OK;
}

ccf_status ccf_batch_submit(ccf_handle** handles, int n, int verbose, ccf_batch** out)
{
	if (!handles || n < 1 || !out) return CCF_ERR_INVALID_ARGUMENT;
	for (int i = 0; i < n; i++)
		if (!handles[i]) return CCF_ERR_INVALID_ARGUMENT;
	ccf_batch* b = new (std::nothrow) ccf_batch();
	if (!b) return CCF_ERR_OUT_OF_MEMORY;
	std::vector<ccf_handle*> hs(handles, handles + n);
	b->worker = std::thread([b, hs, verbose]() mutable {
		ccf_status st = ccf_run_batch(hs.data(), (int)hs.size(), verbose);
		std::lock_guard<std::mutex> g(b->mu);
		b->status = st;
		b->done = true;
		b->cv.notify_all();
	});
	*out = b;
	return CCF_OK;
}

ccf_status ccf_batch_poll(ccf_batch* b, int* done)
{
	if (!b || !done) return CCF_ERR_INVALID_ARGUMENT;
	std::lock_guard<std::mutex> g(b->mu);
	*done = b->done ? 1 : 0;
	return CCF_OK;
}

ccf_status ccf_batch_wait(ccf_batch* b)
{
	if (!b) return CCF_ERR_INVALID_ARGUMENT;
	std::unique_lock<std::mutex> lk(b->mu);
	b->cv.wait(lk, [b] { return b->done; });
	return b->status;
}

void ccf_batch_destroy(ccf_batch* b)
{
	if (!b) return;
	if (b->worker.joinable()) b->worker.join();
	delete b;
}

ccf_status ccf_server_create(const ccf_server_config* cfg, ccf_server** out)
{
	if (!cfg || !out || cfg->slots < 1 || cfg->slots > 64 || cfg->hbm_budget == 0 || cfg->device < 0)
		return CCF_ERR_INVALID_ARGUMENT;
	ccf_server* s = new (std::nothrow) ccf_server();
	if (!s) return CCF_ERR_OUT_OF_MEMORY;
	s->cfg = *cfg;
	s->t0 = std::chrono::steady_clock::now();
	for (int i = 0; i < cfg->slots; i++) s->workers.emplace_back(server_worker, s);
	*out = s;
	return CCF_OK;
}

ccf_status ccf_server_submit(ccf_server* s, const ccf_params* p, long long* id)
{
	if (!s || !p || !id) return CCF_ERR_INVALID_ARGUMENT;
	ccf::Derived d;
	std::string msg;
	if (!derive(*p, d, msg)) return p->starfile[0] ? CCF_ERR_IO : CCF_ERR_INVALID_ARGUMENT;
	std::unique_ptr<ServerRequest> r(new ServerRequest());
	r->params = *p;
	r->bytes = estimate_bytes(*p, d);
	std::lock_guard<std::mutex> g(s->mu);
	if (s->stop) return CCF_ERR_INVALID_ARGUMENT;
	r->id = s->next_id++;
	r->t_submit = now_seconds(s->t0);
	*id = r->id;
	s->queue.push_back(r->id);
	s->reqs[r->id] = std::move(r);
	s->submitted++;
	s->cv_work.notify_all();
	return CCF_OK;
}

ccf_status ccf_server_wait(ccf_server* s, long long id, double timeout_seconds)
{
	if (!s) return CCF_ERR_INVALID_ARGUMENT;
	std::unique_lock<std::mutex> lk(s->mu);
	auto it = s->reqs.find(id);
	if (it == s->reqs.end()) return CCF_ERR_INVALID_ARGUMENT;
	ServerRequest* r = it->second.get();
	auto finished = [r] { return r->state >= CCF_REQUEST_DONE; };
	if (timeout_seconds < 0) s->cv_done.wait(lk, finished);
	else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_seconds), finished)) return CCF_ERR_TIMEOUT;
	return r->status;
}

ccf_status ccf_server_request_info(ccf_server* s, long long id, ccf_request_info* out)
{
	if (!s || !out) return CCF_ERR_INVALID_ARGUMENT;
	std::lock_guard<std::mutex> g(s->mu);
	auto it = s->reqs.find(id);
	if (it == s->reqs.end()) return CCF_ERR_INVALID_ARGUMENT;
	const ServerRequest* r = it->second.get();
	std::memset(out, 0, sizeof(*out));
	out->state = r->state;
	out->status = r->status;
	out->deferred = r->deferred ? 1 : 0;
	out->bytes = r->bytes;
	out->t_submit = r->t_submit;
	out->t_start = r->t_start;
	out->t_end = r->t_end;
	return CCF_OK;
}

ccf_status ccf_server_handle(ccf_server* s, long long id, ccf_handle** h)
{
	if (!s || !h) return CCF_ERR_INVALID_ARGUMENT;
	std::lock_guard<std::mutex> g(s->mu);
	auto it = s->reqs.find(id);
	if (it == s->reqs.end()) return CCF_ERR_INVALID_ARGUMENT;
	const ServerRequest* r = it->second.get();
	if (r->state < CCF_REQUEST_DONE) return CCF_ERR_NOT_RUN;
	if (!r->handle) return r->status == CCF_OK ? CCF_ERR_NOT_RUN : r->status;
	*h = r->handle;
	return CCF_OK;
}

ccf_status ccf_server_release(ccf_server* s, long long id)
{
	if (!s) return CCF_ERR_INVALID_ARGUMENT;
	ccf_handle* h = nullptr;
	{
		std::lock_guard<std::mutex> g(s->mu);
		auto it = s->reqs.find(id);
		if (it == s->reqs.end()) return CCF_ERR_INVALID_ARGUMENT;
		ServerRequest* r = it->second.get();
		if (r->state < CCF_REQUEST_DONE) return CCF_ERR_NOT_RUN;
		h = r->handle;
		r->handle = nullptr;
		if (r->counted)
		{
			s->bytes_in_use -= r->bytes;
			r->counted = false;
		}
	}
	/* free the device memory outside the lock, then let waiting requests in */
	ccf_destroy(h);
	{
		std::lock_guard<std::mutex> g(s->mu);
		s->reqs.erase(id);
		s->cv_work.notify_all();
	}
	return CCF_OK;
}

ccf_status ccf_server_get_stats(ccf_server* s, ccf_server_stats* out)
{
	if (!s || !out) return CCF_ERR_INVALID_ARGUMENT;
	std::lock_guard<std::mutex> g(s->mu);
	std::memset(out, 0, sizeof(*out));
	out->submitted = s->submitted;
	out->admitted = s->admitted;
	out->completed = s->completed;
	out->failed = s->failed;
	out->rejected = s->rejected;
	out->deferred = s->deferred;
	out->queued = (long long)s->queue.size();
	out->running = s->running;
	out->bytes_in_use = s->bytes_in_use;
	out->hbm_budget = s->cfg.hbm_budget;
	return CCF_OK;
}

void ccf_server_destroy(ccf_server* s)
{
	if (!s) return;
	{
		std::lock_guard<std::mutex> g(s->mu);
		s->stop = true;
		s->queue.clear();
		s->cv_work.notify_all();
	}
	for (auto& t : s->workers) t.join();
	for (auto& kv : s->reqs) ccf_destroy(kv.second->handle);
	delete s;
}

} /* extern "C" */
