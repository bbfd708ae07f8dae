// Continuous-batching request server over the batched engine.
//
// Requests (one scene each, with a horizon in steps) queue on submit.  The
// serving loop admits queued requests in arrival order while the HBM budget
// and the arena allow, advances every resident scene by one step per
// substep (one batched launch sequence), and evicts a scene when it reaches
// its horizon or reports non-finite positions.  New requests join between
// substeps, so work from different requests overlaps on the device.  When no
// resident scene reaches its horizon sooner, up to kMaxBurst steps run back
// to back between host checks (the device-side flags accumulate), so the
// host round trip is paid once per burst.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pbf_engine.h"

using namespace pbf103;

namespace {
constexpr uint32_t kMaxBurst = 8;

struct Request {
    uint64_t id = 0;
    pbf_request_desc desc{};
    std::vector<float> x, v;
    uint32_t n = 0;
    uint64_t bytes = 0;
    double arrival = 0, admit = 0, complete = 0;
    uint32_t steps = 0;
    uint32_t scene = UINT32_MAX;
    bool done = false;
    uint32_t flags = 0;
    uint32_t rnum = 0;
    std::vector<float> rx, rv;
    std::unique_ptr<pbf_boundary_t> bnd;
};
}  // namespace

struct pbf_server {
    pbf_server_config cfg{};
    Batch batch;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<uint64_t> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<Request *> resident;
    std::deque<pbf_completion> completions;
    uint64_t next_id = 1;
    pbf_server_stats st{};
    uint64_t resident_bytes = 0;
    std::thread worker;
    bool running = false, stop = false, drain = true;
    pbf_status worker_status = PBF_SUCCESS;
    cudaStream_t stream = nullptr;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    std::vector<uint32_t> nums, flags;

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    // one admit / step / evict round; returns false when there was nothing to do
    pbf_status service(bool *did_work);
    void loop();
};

pbf_status pbf_server::service(bool *did_work)
{
    NvtxRange range("pbf serve round");
    *did_work = false;
    // admit in arrival order while the budget and the arena allow
    for (;;) {
        Request *r = nullptr;
        {
            std::lock_guard<std::mutex> lk(mu);
            if (queue.empty()) break;
            Request *h = reqs[queue.front()].get();
            if (resident_bytes + h->bytes > cfg.hbm_budget_bytes) break;
            queue.pop_front();
            r = h;
        }
        const float *de = r->desc.domain_end;
        uint32_t id = 0;
        const uint32_t cap = r->desc.capacity ? r->desc.capacity : r->n;
        pbf_status rc = batch.add_scene(r->desc.params, cap, de, r->bnd.get(), r->desc.area_min, r->desc.area_max,
                                        r->x.data(), r->v.data(), r->n, false, stream, &id);
        std::lock_guard<std::mutex> lk(mu);
        if ((rc == PBF_ERROR_OUT_OF_MEMORY || rc == PBF_ERROR_CAPACITY) && !resident.empty()) {
            // arena full or fragmented: retry after the next eviction
            queue.push_front(r->id);
            break;
        }
        if (rc != PBF_SUCCESS) {  // refused, or too large even for the arena with nothing resident
            r->done = true;
            r->complete = now();
            r->flags = 0xFFFFFFFFu;
            st.rejected++;
            pbf_completion c{r->id, 0, 0, r->flags, r->arrival, r->complete, r->complete};
            completions.push_back(c);
            *did_work = true;
            continue;
        }
        r->scene = id;
        r->admit = now();
        r->x.clear();
        r->x.shrink_to_fit();
        r->v.clear();
        r->v.shrink_to_fit();
        resident_bytes += r->bytes;
        st.admitted++;
        if (resident_bytes > st.peak_resident_bytes) st.peak_resident_bytes = resident_bytes;
        resident.push_back(r);
        *did_work = true;
    }
    if (resident.empty()) return PBF_SUCCESS;

    // steps until the first resident scene reaches its horizon, at most kMaxBurst
    uint32_t burst = kMaxBurst;
    for (Request *r : resident) burst = std::min(burst, r->desc.horizon_steps - r->steps);
    burst = std::max(burst, 1u);
    const double t_step = now();
    for (uint32_t k = 0; k < burst; ++k) {
        pbf_status rc = batch.step(cfg.iters, stream);
        if (rc != PBF_SUCCESS) return rc;
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess) return PBF_ERROR_CUDA;
    const double t_done = now();
    *did_work = true;

    std::vector<Request *> keep;
    keep.reserve(resident.size());
    uint64_t ps = 0;
    pbf_status rc = batch.read_all(nums, flags, true, stream);
    if (rc != PBF_SUCCESS) return rc;
    for (Request *r : resident) {
        const uint32_t n = nums[r->scene], f = flags[r->scene];
        ps += (uint64_t)n * burst;  // live count after the burst (deletions only lower it)
        r->steps += burst;
        r->flags |= f;
        const bool finished = r->steps >= r->desc.horizon_steps || (f & PBF_FLAG_NONFINITE);
        if (!finished) {
            keep.push_back(r);
            continue;
        }
        r->rx.resize(3ull * n);
        r->rv.resize(3ull * n);
        uint32_t num = 0;
        batch.get_particles(r->scene, r->rx.data(), r->rv.data(), &num, false, stream);
        r->rnum = num;
        batch.remove_scene(r->scene);
        std::lock_guard<std::mutex> lk(mu);
        r->done = true;
        r->complete = now();
        resident_bytes -= r->bytes;
        st.completed++;
        pbf_completion c{r->id, r->rnum, r->steps, r->flags, r->arrival, r->admit, r->complete};
        completions.push_back(c);
    }
    std::lock_guard<std::mutex> lk(mu);
    resident.swap(keep);
    st.substeps += burst;
    st.particle_steps += ps;
    st.busy_s += t_done - t_step;
    return PBF_SUCCESS;
}

void pbf_server::loop()
{
    cudaSetDevice(cfg.device);
    for (;;) {
        bool worked = false;
        pbf_status rc = service(&worked);
        if (rc != PBF_SUCCESS) {
            std::lock_guard<std::mutex> lk(mu);
            worker_status = rc;
            running = false;
            cv.notify_all();
            return;
        }
        std::unique_lock<std::mutex> lk(mu);
        if (stop && (!drain || (queue.empty() && resident.empty()))) break;
        if (!worked) cv.wait_for(lk, std::chrono::milliseconds(1));
    }
    std::lock_guard<std::mutex> lk(mu);
    running = false;
    cv.notify_all();
}

extern "C" {

pbf_status pbf_server_create(const pbf_server_config *cfg, pbf_server **out)
{
    if (!cfg || !out || cfg->iters < 0) return PBF_ERROR_INVALID_ARGUMENT;
    std::unique_ptr<pbf_server> s(new (std::nothrow) pbf_server());
    if (!s) return PBF_ERROR_OUT_OF_MEMORY;
    s->cfg = *cfg;
    if (!s->cfg.max_pair) s->cfg.max_pair = 30;
    pbf_status rc = s->batch.init(cfg->max_scenes, cfg->max_particles, cfg->max_cells, s->cfg.max_pair, cfg->device);
    if (rc != PBF_SUCCESS) return rc;
    if (cfg->tile) {
        rc = s->batch.set_tile(cfg->tile);
        if (rc != PBF_SUCCESS) return rc;
    }
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return PBF_ERROR_CUDA;
    s->t0 = std::chrono::steady_clock::now();
    *out = s.release();
    return PBF_SUCCESS;
}

pbf_status pbf_server_destroy(pbf_server *s)
{
    if (!s) return PBF_SUCCESS;
    pbf_server_stop(s, 0);
    cudaSetDevice(s->cfg.device);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return PBF_SUCCESS;
}

pbf_status pbf_server_submit(pbf_server *s, const pbf_request_desc *req, const float *x, const float *v, uint32_t n,
                             uint64_t *request_id)
{
    if (!s || !req || !request_id || (n && !x) || req->n_planes > 8 || req->horizon_steps == 0)
        return PBF_ERROR_INVALID_ARGUMENT;
    const uint32_t cap = req->capacity ? req->capacity : n;
    if (cap < n || cap == 0) return PBF_ERROR_INVALID_ARGUMENT;
    uint64_t bytes = 0;
    pbf_status rc = pbf_scene_bytes(&req->params, cap, req->domain_end, &bytes);
    if (rc != PBF_SUCCESS) return rc;
    SceneDesc d;
    uint32_t grid[3];
    rc = derive_desc(req->params, req->domain_end, &d, grid);
    if (rc != PBF_SUCCESS) return rc;
    std::unique_ptr<Request> r(new (std::nothrow) Request());
    if (!r) return PBF_ERROR_OUT_OF_MEMORY;
    r->desc = *req;
    r->n = n;
    r->bytes = bytes;
    r->x.assign(x, x + 3ull * n);
    if (v) r->v.assign(v, v + 3ull * n);
    else r->v.assign(3ull * n, 0.f);
    if (req->n_planes) {
        pbf_boundary_t *b = nullptr;
        rc = pbf_boundary_create(nullptr, 0, nullptr, 0, &req->plane_points[0][0], &req->plane_normals[0][0],
                                 req->n_planes, &b);
        if (rc != PBF_SUCCESS) return rc;
        r->bnd.reset(b);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->st.submitted++;
    if (bytes > s->cfg.hbm_budget_bytes) {
        s->st.rejected++;
        return PBF_ERROR_BUDGET;
    }
    // a request larger than the empty arena would wait forever at the head of
    // the queue: refuse it here
    if (!s->batch.ever_fits(cap, (uint64_t)d.ncell + 1)) {
        s->st.rejected++;
        return PBF_ERROR_CAPACITY;
    }
    r->id = s->next_id++;
    r->arrival = s->now();
    *request_id = r->id;
    s->queue.push_back(r->id);
    s->reqs.emplace(r->id, std::move(r));
    s->cv.notify_all();
    return PBF_SUCCESS;
}

pbf_status pbf_server_start(pbf_server *s)
{
    if (!s) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->running) return PBF_SUCCESS;
    s->stop = false;
    s->running = true;
    s->worker_status = PBF_SUCCESS;
    s->worker = std::thread([s] { s->loop(); });
    return PBF_SUCCESS;
}

pbf_status pbf_server_stop(pbf_server *s, int drain)
{
    if (!s) return PBF_ERROR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->drain = drain != 0;
        s->cv.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    return s->worker_status;
}

pbf_status pbf_server_run_until_idle(pbf_server *s)
{
    if (!s) return PBF_ERROR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->running) return PBF_ERROR_INVALID_ARGUMENT;
    }
    cudaSetDevice(s->cfg.device);
    for (;;) {
        bool worked = false;
        pbf_status rc = s->service(&worked);
        if (rc != PBF_SUCCESS) return rc;
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->queue.empty() && s->resident.empty()) return PBF_SUCCESS;
        if (!worked && s->resident.empty()) return PBF_ERROR_CAPACITY;  // head request can never fit
    }
}

pbf_status pbf_server_poll(pbf_server *s, pbf_completion *out, uint32_t max, uint32_t *n_out)
{
    if (!s || !n_out || (max && !out)) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    uint32_t k = 0;
    while (k < max && !s->completions.empty()) {
        out[k++] = s->completions.front();
        s->completions.pop_front();
    }
    *n_out = k;
    return PBF_SUCCESS;
}

pbf_status pbf_server_result(pbf_server *s, uint64_t id, float *x, float *v, uint32_t *num)
{
    if (!s) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return PBF_ERROR_NOT_FOUND;
    Request *r = it->second.get();
    if (!r->done) return PBF_ERROR_NOT_READY;
    if (num) *num = r->rnum;
    if (x && r->rnum) std::memcpy(x, r->rx.data(), 12ull * r->rnum);
    if (v && r->rnum) std::memcpy(v, r->rv.data(), 12ull * r->rnum);
    return PBF_SUCCESS;
}

pbf_status pbf_server_release(pbf_server *s, uint64_t id)
{
    if (!s) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return PBF_ERROR_NOT_FOUND;
    if (!it->second->done) return PBF_ERROR_NOT_READY;
    s->reqs.erase(it);
    return PBF_SUCCESS;
}

pbf_status pbf_server_get_stats(pbf_server *s, pbf_server_stats *out)
{
    if (!s || !out) return PBF_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->resident_bytes = s->resident_bytes;
    out->resident_scenes = (uint32_t)s->resident.size();
    out->queued = (uint32_t)s->queue.size();
    out->elapsed_s = s->now();
    return PBF_SUCCESS;
}

double pbf_server_clock(pbf_server *s) { return s ? s->now() : 0.0; }

}  // extern "C"
