// Request server (cs_server_*): continuous batching of build + neighbour-query requests and incremental updates of
// resident trees on one GPU.
//
// A request is a particle set (host arrays) with a box: BUILD computes keys -> sort -> tree -> link -> geometry ->
// neighbours from the root; with a tree id the result stays resident on the device; UPDATE applies one
// updateOctree step of a resident tree to new positions of its particles (the reference's per-time-step path). Each
// of num_slots worker threads owns a CUDA stream and a pipeline object and takes the oldest admissible request:
// the first queued request of its tree (requests of one tree run in order, one at a time) whose device memory fits
// the budget. Requests that arrive while others run are admitted as slots and memory free up, so the work of
// several requests overlaps on the device. Memory: the sum of the device bytes of every pipeline (slots and resident
// trees) plus the growth an admitted request may need; a request that does not fit waits, least recently used idle
// resident trees are released to make room, and a request that cannot fit even on an idle server fails
// (CS_ERR_CAPACITY). Each result (leaf count, neighbour counts, a checksum of the neighbour lists) depends only on
// the request's own inputs, so it is the same alone and in any mix.
#include "cs_common.cuh"
#include "pipeline.cuh"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace csg
{

using Clock = std::chrono::steady_clock;

static double msSince(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request
{
    uint64_t id = 0;
    cs_request r{};
    Clock::time_point submitted;
};

struct Result
{
    cs_request_result res{};
    std::vector<uint32_t> nc;
    bool done = false;
};

struct Tree
{
    std::unique_ptr<PipelineBase> pipe;
    DevBuf x, y, z, h; // device copies of the positions, stable across updates
    size_t n      = 0;
    bool busy     = false;
    bool built    = false;
    uint64_t used = 0; // last use, for least-recently-used release
};

struct Server
{
    cs_server_config cfg{};
    std::mutex m;
    std::condition_variable cvWork, cvDone;
    std::deque<Request> queue;
    std::map<uint64_t, Result> results;
    std::map<int32_t, Tree> trees;
    std::vector<std::unique_ptr<PipelineBase>> slotPipes;
    std::vector<cudaStream_t> streams;
    std::vector<std::thread> workers;
    std::vector<size_t> slotBytes; // device bytes of each idle slot's pipeline (0 while it runs a request)
    std::vector<char> slotBusy;
    size_t treeBytes     = 0;
    size_t reserved      = 0; // growth promised to running requests
    uint64_t nextId      = 1;
    uint64_t useClock    = 0;
    int running          = 0;
    bool stop            = false;
    int device           = 0;
    std::vector<double> latencies;
    uint64_t completed = 0, failed = 0, particles = 0;
    Clock::time_point firstSubmit{}, lastDone{};
    bool anySubmit = false;

    // device bytes a pipeline needs for n particles (an upper estimate of what it grows to)
    size_t estimate(size_t n) const
    {
        size_t coord = cfg.coord_bits == 64 ? 8 : 4, key = cfg.key_bits == 64 ? 8 : 4;
        size_t perParticle = 4 * coord * 3 + 2 * key + 8 + 32 + 16 * 2 + 4 * cfg.pipeline.ngmax + 8;
        size_t leaves      = n / std::max(1u, cfg.pipeline.bucket_size) * 8 + 4096;
        return n * perParticle + leaves * (3 * (key + 4) + 6 * coord + 64) + (size_t(64) << 20);
    }

    size_t used() const
    {
        size_t t = treeBytes + reserved;
        for (size_t b : slotBytes)
            t += b;
        return t;
    }

    // index of the queued request a free slot may run now, or -1; releases idle resident trees to make room
    int pick(int slot, int* failIdx)
    {
        *failIdx = -1;
        std::map<int32_t, bool> seenTree;
        for (size_t q = 0; q < queue.size(); ++q)
        {
            const cs_request& r = queue[q].r;
            if (r.tree >= 0)
            {
                if (seenTree.count(r.tree)) continue; // an earlier request of this tree goes first
                seenTree[r.tree] = true;
                auto it          = trees.find(r.tree);
                if (it != trees.end() && it->second.busy) continue;
                if (r.kind == CS_REQ_UPDATE && (it == trees.end() || !it->second.built || it->second.n != r.n))
                {
                    *failIdx = int(q); // nothing to update
                    return -1;
                }
            }
            size_t need = estimate(r.n);
            size_t have = r.tree >= 0 && trees.count(r.tree) ? trees[r.tree].pipe->deviceBytes() : slotBytes[slot];
            size_t grow = need > have ? need - have : 0;
            while (used() + grow > cfg.hbm_budget_bytes)
            {
                // release the least recently used idle resident tree (not the one this request needs)
                int32_t victim = -1;
                uint64_t best  = ~0ull;
                for (auto& kv : trees)
                    if (!kv.second.busy && kv.first != r.tree && kv.second.used < best)
                    {
                        best   = kv.second.used;
                        victim = kv.first;
                    }
                if (victim < 0) break;
                treeBytes -= trees[victim].pipe->deviceBytes();
                trees.erase(victim);
            }
            for (size_t k = 0; k < slotPipes.size() && used() + grow > cfg.hbm_budget_bytes; ++k)
            {
                // then the buffers that other idle slots grew for earlier requests
                if (int(k) == slot || slotBusy[k] || slotBytes[k] == 0) continue;
                slotPipes[k] = makePipeline(cfg.coord_bits, cfg.key_bits, cfg.pipeline);
                slotBytes[k] = 0;
            }
            if (used() + grow <= cfg.hbm_budget_bytes) return int(q);
            if (running == 0)
            {
                *failIdx = int(q); // does not fit even on an idle server
                return -1;
            }
            return -1; // wait for memory, in arrival order
        }
        return -1;
    }

    void finish(const Request& rq, int status, int32_t leaves, uint64_t checksum, std::vector<uint32_t>&& nc,
                Clock::time_point started)
    {
        Clock::time_point now = Clock::now();
        Result& out           = results[rq.id];
        out.res.id                = rq.id;
        out.res.status            = status;
        out.res.num_leaves        = leaves;
        out.res.neighbor_checksum = checksum;
        out.res.queued_ms         = msSince(rq.submitted, started);
        out.res.run_ms            = msSince(started, now);
        out.res.latency_ms        = msSince(rq.submitted, now);
        out.nc                    = std::move(nc);
        out.done                  = true;
        if (status == CS_OK)
        {
            completed++;
            particles += rq.r.n;
            latencies.push_back(out.res.latency_ms);
        }
        else failed++;
        lastDone = now;
        cvDone.notify_all();
    }

    void worker(int slot)
    {
        cudaSetDevice(device);
        cudaStream_t s = streams[slot];
        std::unique_lock<std::mutex> lk(m);
        for (;;)
        {
            int failIdx = -1, q = -1;
            cvWork.wait(lk, [&] {
                if (stop && queue.empty()) return true;
                q = pick(slot, &failIdx);
                return q >= 0 || failIdx >= 0;
            });
            if (q < 0 && failIdx < 0) return; // stopping, queue drained
            if (failIdx >= 0)
            {
                Request rq = queue[failIdx];
                queue.erase(queue.begin() + failIdx);
                setLastError("server: request %llu cannot run (no resident tree to update, or over the budget)",
                             (unsigned long long)rq.id);
                finish(rq, rq.r.kind == CS_REQ_UPDATE ? CS_ERR_INVALID : CS_ERR_CAPACITY, 0, 0, {}, Clock::now());
                continue;
            }
            Request rq = queue[q];
            queue.erase(queue.begin() + q);
            const cs_request& r = rq.r;
            Tree* tree          = nullptr;
            if (r.tree >= 0)
            {
                Tree& t = trees[r.tree]; // created on first use
                if (!t.pipe) t.pipe = makePipeline(cfg.coord_bits, cfg.key_bits, cfg.pipeline);
                t.busy  = true;
                t.used  = ++useClock;
                treeBytes -= t.pipe->deviceBytes();
                tree = &t;
            }
            // while it runs, the request holds what its pipeline may grow to
            const size_t before = tree ? tree->pipe->deviceBytes() : slotBytes[slot];
            const size_t hold   = std::max(estimate(r.n), before);
            if (!tree)
            {
                slotBytes[slot] = 0;
                slotBusy[slot]  = 1;
            }
            reserved += hold;
            running++;
            Clock::time_point started = Clock::now();
            lk.unlock();

            // ---- run the request on this slot's stream ----
            int status = CS_OK;
            int32_t leaves = 0;
            uint64_t checksum = 0;
            std::vector<uint32_t> nc;
            PipelineBase* pipe = tree ? tree->pipe.get() : slotPipes[slot].get();
            cs_pipeline_result pr{};
            const size_t coord = cfg.coord_bits == 64 ? 8 : 4;
            if (tree)
            {
                // resident tree: positions into its stable device buffers, then a root build or one update step
                for (DevBuf* b : {&tree->x, &tree->y, &tree->z, &tree->h})
                    if (!status) status = b->ensure(r.n * coord);
                const void* src[4] = {r.x, r.y, r.z, r.h};
                DevBuf* dst[4]     = {&tree->x, &tree->y, &tree->z, &tree->h};
                for (int k = 0; k < 4 && !status; ++k)
                    if (cudaMemcpyAsync(dst[k]->p, src[k], r.n * coord, cudaMemcpyHostToDevice, s) != cudaSuccess)
                        status = CS_ERR_CUDA;
                if (!status)
                {
                    if (r.kind == CS_REQ_BUILD) pipe->resetSteps();
                    status = pipe->step(s, tree->x.p, tree->y.p, tree->z.p, tree->h.p, r.n, r.box, false, &pr);
                }
                if (!status)
                {
                    tree->n     = r.n;
                    tree->built = true;
                }
            }
            else status = pipe->run(s, r.x, r.y, r.z, r.h, r.n, r.box, 0, 0, &pr, true);
            if (!status)
            {
                leaves = pr.num_leaves;
                cs_pipeline_outputs o{};
                pipe->outputs(&o);
                nc.resize(r.n);
                if (cudaMemcpyAsync(nc.data(), o.neighbor_counts, r.n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s) !=
                    cudaSuccess)
                    status = CS_ERR_CUDA;
                if (!status && o.neighbors)
                {
                    DevBuf scratch;
                    if (scratch.ensure(sizeof(uint64_t)) == CS_OK)
                        checksum = neighborChecksum(s, o.neighbors, o.neighbor_counts, r.n, cfg.pipeline.ngmax,
                                                    scratch.as<uint64_t>());
                }
                if (cudaStreamSynchronize(s) != cudaSuccess) status = CS_ERR_CUDA;
            }

            lk.lock();
            running--;
            reserved -= hold;
            if (tree)
            {
                tree->busy = false;
                treeBytes += tree->pipe->deviceBytes();
                if (status && !tree->built)
                {
                    treeBytes -= tree->pipe->deviceBytes();
                    trees.erase(r.tree);
                }
            }
            else
            {
                slotBytes[slot] = pipe->deviceBytes();
                slotBusy[slot]  = 0;
            }
            finish(rq, status, leaves, checksum, std::move(nc), started);
            cvWork.notify_all();
        }
    }
};

} // namespace csg

using namespace csg;

struct cs_server_s
{
    std::unique_ptr<Server> impl;
};

extern "C" int cs_server_create(cs_server* out, const cs_server_config* cfg)
{
    if (!out || !cfg || cfg->num_slots < 1 || cfg->num_slots > 64 || (cfg->coord_bits != 32 && cfg->coord_bits != 64) ||
        (cfg->key_bits != 32 && cfg->key_bits != 64) || cfg->pipeline.bucket_size == 0)
    {
        setLastError("server create: invalid arguments");
        return CS_ERR_INVALID;
    }
    auto sv  = std::make_unique<Server>();
    sv->cfg  = *cfg;
    CSG_CUDA_TRY(cudaGetDevice(&sv->device));
    int n = cfg->num_slots;
    sv->streams.resize(n);
    sv->slotBytes.assign(n, 0);
    sv->slotBusy.assign(n, 0);
    for (int k = 0; k < n; ++k)
    {
        CSG_CUDA_TRY(cudaStreamCreateWithFlags(&sv->streams[k], cudaStreamNonBlocking));
        cs_pipeline_config pc = cfg->pipeline;
        pc.do_halos           = 0;
        sv->slotPipes.push_back(makePipeline(cfg->coord_bits, cfg->key_bits, pc));
    }
    sv->cfg.pipeline.do_halos = 0;
    Server* raw = sv.get();
    for (int k = 0; k < n; ++k)
        sv->workers.emplace_back([raw, k] { raw->worker(k); });
    auto* s = new cs_server_s;
    s->impl = std::move(sv);
    *out    = s;
    return CS_OK;
}

extern "C" int cs_server_destroy(cs_server s)
{
    if (!s) return CS_OK;
    Server* sv = s->impl.get();
    {
        std::lock_guard<std::mutex> lk(sv->m);
        sv->stop = true;
    }
    sv->cvWork.notify_all();
    for (auto& t : sv->workers)
        t.join();
    sv->slotPipes.clear();
    sv->trees.clear();
    for (cudaStream_t st : sv->streams)
        cudaStreamDestroy(st);
    delete s;
    return CS_OK;
}

extern "C" int cs_server_submit(cs_server s, const cs_request* req, uint64_t* id)
{
    if (!s || !req || !req->x || !req->y || !req->z || !req->h || req->n == 0 || req->n >= (size_t(1) << 30) ||
        (req->kind != CS_REQ_BUILD && req->kind != CS_REQ_UPDATE) || (req->kind == CS_REQ_UPDATE && req->tree < 0))
    {
        setLastError("server submit: invalid request");
        return CS_ERR_INVALID;
    }
    Server* sv = s->impl.get();
    {
        std::lock_guard<std::mutex> lk(sv->m);
        if (sv->stop)
        {
            setLastError("server submit: server is stopping");
            return CS_ERR_INVALID;
        }
        Request rq;
        rq.id        = sv->nextId++;
        rq.r         = *req;
        rq.submitted = Clock::now();
        if (!sv->anySubmit)
        {
            sv->anySubmit   = true;
            sv->firstSubmit = rq.submitted;
        }
        sv->results[rq.id] = Result{};
        sv->queue.push_back(rq);
        if (id) *id = rq.id;
    }
    sv->cvWork.notify_all();
    return CS_OK;
}

extern "C" int cs_server_wait(cs_server s, uint64_t id, cs_request_result* res, uint32_t* ncHost)
{
    if (!s)
    {
        setLastError("server wait: null server");
        return CS_ERR_INVALID;
    }
    Server* sv = s->impl.get();
    std::unique_lock<std::mutex> lk(sv->m);
    auto it = sv->results.find(id);
    if (it == sv->results.end())
    {
        setLastError("server wait: unknown request %llu", (unsigned long long)id);
        return CS_ERR_INVALID;
    }
    sv->cvDone.wait(lk, [&] { return sv->results[id].done; });
    Result r = std::move(sv->results[id]);
    sv->results.erase(id);
    lk.unlock();
    if (res) *res = r.res;
    if (ncHost && !r.nc.empty()) std::memcpy(ncHost, r.nc.data(), r.nc.size() * sizeof(uint32_t));
    return r.res.status;
}

extern "C" int cs_server_release_tree(cs_server s, int32_t tree)
{
    if (!s)
    {
        setLastError("server release: null server");
        return CS_ERR_INVALID;
    }
    Server* sv = s->impl.get();
    std::unique_lock<std::mutex> lk(sv->m);
    auto it = sv->trees.find(tree);
    if (it == sv->trees.end()) return CS_OK;
    if (it->second.busy)
    {
        setLastError("server release: tree %d is in use", tree);
        return CS_ERR_INVALID;
    }
    sv->treeBytes -= it->second.pipe->deviceBytes();
    sv->trees.erase(it);
    sv->cvWork.notify_all();
    return CS_OK;
}

extern "C" int cs_server_get_stats(cs_server s, cs_server_stats* st)
{
    if (!s || !st)
    {
        setLastError("server stats: null argument");
        return CS_ERR_INVALID;
    }
    Server* sv = s->impl.get();
    std::lock_guard<std::mutex> lk(sv->m);
    std::vector<double> l = sv->latencies;
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, size_t(p * double(l.size())))]; };
    st->completed      = sv->completed;
    st->failed         = sv->failed;
    st->particles      = sv->particles;
    st->p50_ms         = pct(0.50);
    st->p99_ms         = pct(0.99);
    st->elapsed_s      = sv->anySubmit ? msSince(sv->firstSubmit, sv->lastDone) * 1e-3 : 0.0;
    st->device_bytes   = sv->used();
    st->resident_trees = int(sv->trees.size());
    return CS_OK;
}
