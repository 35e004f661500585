// server.cu -- the continuous-batching request loop (host C++), written on
// top of the library's own batch C ABI.
//
// Galaxy's serving front ends render one request at a time
// (ViewerClientServer::handle `render`, multiserver/ViewerClientServer.cpp:
// 62-253; GuiClientServer gui::render, guiserver/GuiClientServer.cpp:375-407)
// and stream pixels per ServerRendering::AddLocalPixels
// (ServerRendering.cpp:45-66).  Here a worker thread keeps several batch
// slots (each a gxy_batch with its own stream) busy:
//   * a submitted request waits in arrival order;
//   * whenever a slot is free, requests up to small_pixels are packed -- same
//     scene, oldest first -- into one batch of at most small_batch_pixels, and
//     a larger request gets a slot of its own; small requests may pass a
//     large one that has waited less than big_wait_s;
//   * a request is admitted only while its framebuffer fits the framebuffer
//     budget; framebuffers come from a stream-ordered CUDA memory pool, so
//     taking and returning them never synchronises the device;
//   * completions are found by polling the slots; a finished request keeps
//     its framebuffer until the client takes the image.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gxy_host.h"

namespace gxy {

namespace {

enum { R_WAITING = 0, R_RUNNING = 1, R_DONE = 2, R_FAILED = 3 };

struct SReq {
    gxy_scene scene = nullptr;
    gxy_camera cam{};
    gxy_lighting light{};
    int64_t pixels = 0;
    double arrival = 0, t_done = -1;
    float *fb = nullptr;
    size_t fb_bytes = 0;
    int64_t rays = 0;
    int state = R_WAITING;
    bool cancel = false;                // cancelled while running: the result is discarded
    int error = GXY_OK;
    std::string message;
};

struct Slot {
    gxy_batch batch = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<int64_t> ids;
};

}  // namespace

struct Server {
    gxy_server_config cfg{};
    int device = 0;
    std::vector<Slot> slots;
    cudaMemPool_t pool = nullptr;
    cudaStream_t io = nullptr;          // image copies out and framebuffer returns
    std::mutex mu;
    std::condition_variable cv;         // a request finished
    std::deque<int64_t> waiting;
    std::unordered_map<int64_t, SReq> reqs;
    size_t fb_used = 0;
    int64_t next_id = 1, pending = 0;   // submitted and not finished
    std::atomic<bool> stop{false};
    std::thread worker;
    std::string worker_error;
    const std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    void finish(Slot &s);
    bool admit(Slot &s);
    void loop();
};

void Server::finish(Slot &s) {
    gxy_counters c{};
    int rc = gxy_gpu_batch_counters(s.batch, &c);
    const double t = now();
    int64_t tot = 0;
    for (int64_t id : s.ids) tot += reqs[id].pixels;
    const int64_t rays = c.primary_rays + c.shadow_rays + c.ao_rays;
    for (int64_t id : s.ids) {
        SReq &r = reqs[id];
        r.t_done = t;
        r.rays = tot ? (int64_t)((double)rays * r.pixels / tot) : 0;
        r.state = (rc == GXY_OK && !r.cancel) ? R_DONE : R_FAILED;
        r.error = r.cancel ? GXY_ERR_CANCELLED : rc;
        if (r.cancel) r.message = "cancelled";
        pending--;
    }
    s.ids.clear();
}

bool Server::admit(Slot &s) {
    if (waiting.empty()) return false;
    const double t = now();
    const SReq &head = reqs[waiting.front()];
    bool small_waiting = false;
    for (int64_t id : waiting)
        if (reqs[id].pixels <= cfg.small_pixels) { small_waiting = true; break; }
    std::vector<int64_t> cand;
    int64_t cap;
    if (head.pixels > cfg.small_pixels && (!small_waiting || t - head.arrival >= cfg.big_wait_s)) {
        cand.push_back(waiting.front());
        cap = cfg.slot_pixels;
    } else {
        gxy_scene key = nullptr;
        for (int64_t id : waiting) {
            const SReq &r = reqs[id];
            if (r.pixels > cfg.small_pixels) continue;
            if (!key) key = r.scene;
            if (r.scene == key) cand.push_back(id);
        }
        cap = std::min(cfg.small_batch_pixels, cfg.slot_pixels);
    }
    std::vector<gxy_job> jobs;
    int64_t pix = 0;
    for (int64_t id : cand) {
        SReq &r = reqs[id];
        if ((int)jobs.size() >= cfg.max_jobs || pix + r.pixels > cap) break;
        const size_t bytes = (size_t)r.pixels * 4 * sizeof(float);
        if (fb_used + bytes > cfg.fb_budget_bytes) break;
        void *p = nullptr;
        if (cudaMallocFromPoolAsync(&p, bytes, pool, s.stream) != cudaSuccess) {
            cudaGetLastError();
            break;
        }
        cudaMemsetAsync(p, 0, bytes, s.stream);   // contributions are added
        r.fb = (float *)p;
        r.fb_bytes = bytes;
        fb_used += bytes;
        gxy_job j{};
        j.scene = r.scene;
        j.camera = r.cam;
        j.lighting = r.light;
        j.fb_rgba = r.fb;
        jobs.push_back(j);
        s.ids.push_back(id);
        pix += r.pixels;
    }
    if (jobs.empty()) return false;
    for (int64_t id : s.ids) {
        waiting.erase(std::find(waiting.begin(), waiting.end(), id));
        reqs[id].state = R_RUNNING;
    }
    const int flags = (cfg.use_graph ? GXY_BATCH_GRAPH : 0) | (cfg.cooperative ? GXY_BATCH_COOPERATIVE : 0);
    int rc = gxy_gpu_batch_submit(s.batch, jobs.data(), (int)jobs.size(), flags);
    if (rc != GXY_OK) {
        std::string msg = last_error();
        for (int64_t id : s.ids) {
            SReq &r = reqs[id];
            r.state = R_FAILED;
            r.error = rc;
            r.message = msg;
            r.t_done = now();
            pending--;
        }
        s.ids.clear();
        cv.notify_all();
        return false;
    }
    return true;
}

void Server::loop() {
    cudaSetDevice(device);
    while (!stop.load()) {
        bool progress = false;
        {
            std::lock_guard<std::mutex> lock(mu);
            for (Slot &s : slots) {
                if (s.ids.empty()) continue;
                int done = 0;
                if (gxy_gpu_batch_poll(s.batch, &done) != GXY_OK) done = 1;   // the error is the batch's status
                if (done) {
                    finish(s);
                    progress = true;
                }
            }
            for (Slot &s : slots)
                if (s.ids.empty() && admit(s)) progress = true;
            if (progress) cv.notify_all();
        }
        if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

}  // namespace gxy

using namespace gxy;

extern "C" {

int gxy_server_create(const gxy_server_config *cfg, gxy_server *out) {
    if (!cfg || !out) return set_error(GXY_ERR_INVALID, "null argument");
    if (cfg->n_slots < 1 || cfg->n_slots > 64 || cfg->slot_pixels <= 0 || cfg->max_jobs < 1)
        return set_error(GXY_ERR_INVALID, "bad server configuration");
    std::unique_ptr<Server> s(new Server());
    s->cfg = *cfg;
    if (s->cfg.small_batch_pixels <= 0) s->cfg.small_batch_pixels = s->cfg.slot_pixels;
    CK(cudaGetDevice(&s->device));
    for (int k = 0; k < cfg->n_slots; k++) {
        Slot sl;
        int rc = gxy_gpu_batch_create(cfg->slot_pixels, cfg->max_jobs, cfg->max_shadow, cfg->max_ao, &sl.batch);
        if (rc != GXY_OK) {
            for (Slot &o : s->slots) gxy_gpu_batch_release(o.batch);
            return rc;
        }
        void *st = nullptr;
        gxy_gpu_batch_stream(sl.batch, &st);
        sl.stream = (cudaStream_t)st;
        s->slots.push_back(sl);
    }
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    CK(cudaMemPoolCreate(&s->pool, &props));
    uint64_t keep = UINT64_MAX;   // returned framebuffers stay in the pool
    CK(cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    CK(cudaStreamCreateWithFlags(&s->io, cudaStreamNonBlocking));
    Server *raw = s.get();
    s->worker = std::thread([raw] { raw->loop(); });
    *out = reinterpret_cast<gxy_server>(s.release());
    return GXY_OK;
}

int gxy_server_release(gxy_server server) {
    if (!server) return set_error(GXY_ERR_INVALID, "null server");
    Server *s = reinterpret_cast<Server *>(server);
    s->stop.store(true);
    if (s->worker.joinable()) s->worker.join();
    for (Slot &sl : s->slots) {
        if (!sl.ids.empty()) gxy_gpu_batch_wait(sl.batch, 60000);
        gxy_gpu_batch_release(sl.batch);
    }
    for (auto &kv : s->reqs)
        if (kv.second.fb) cudaFreeAsync(kv.second.fb, s->io);
    cudaStreamSynchronize(s->io);
    cudaStreamDestroy(s->io);
    cudaMemPoolDestroy(s->pool);
    delete s;
    return GXY_OK;
}

int gxy_server_submit(gxy_server server, gxy_scene scene, const gxy_camera *camera, const gxy_lighting *lighting,
                      int64_t *id) {
    if (!server || !scene || !camera || !lighting || !id) return set_error(GXY_ERR_INVALID, "null argument");
    Server *s = reinterpret_cast<Server *>(server);
    if (camera->width <= 0 || camera->height <= 0) return set_error(GXY_ERR_INVALID, "bad image size");
    const int64_t pixels = (int64_t)camera->width * camera->height;
    if (pixels > s->cfg.slot_pixels) return set_error(GXY_ERR_ADMISSION, "request larger than a batch slot");
    if ((size_t)pixels * 16 > s->cfg.fb_budget_bytes)
        return set_error(GXY_ERR_ADMISSION, "request framebuffer larger than the framebuffer budget");
    std::lock_guard<std::mutex> lock(s->mu);
    SReq r;
    r.scene = scene;
    r.cam = *camera;
    r.light = *lighting;
    r.pixels = pixels;
    r.arrival = s->now();
    *id = s->next_id++;
    s->reqs[*id] = r;
    s->waiting.push_back(*id);
    s->pending++;
    return GXY_OK;
}

int gxy_server_poll(gxy_server server, int64_t id, int *done) {
    if (!server || !done) return set_error(GXY_ERR_INVALID, "null argument");
    Server *s = reinterpret_cast<Server *>(server);
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return set_error(GXY_ERR_INVALID, "unknown request");
    *done = it->second.state >= R_DONE ? 1 : 0;
    return GXY_OK;
}

int gxy_server_cancel(gxy_server server, int64_t id, int *was_running) {
    if (!server) return set_error(GXY_ERR_INVALID, "null server");
    Server *s = reinterpret_cast<Server *>(server);
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return set_error(GXY_ERR_INVALID, "unknown request");
    SReq &r = it->second;
    if (was_running) *was_running = r.state == R_RUNNING;
    if (r.state == R_WAITING) {
        s->waiting.erase(std::find(s->waiting.begin(), s->waiting.end(), id));
        r.state = R_FAILED;
        r.error = GXY_ERR_CANCELLED;
        r.message = "cancelled";
        r.t_done = s->now();
        s->pending--;
        s->cv.notify_all();
    } else if (r.state == R_RUNNING) {
        r.cancel = true;   // its batch runs to the end; the image is discarded
    }
    return GXY_OK;
}

int gxy_server_drain(gxy_server server, int timeout_ms) {
    if (!server) return set_error(GXY_ERR_INVALID, "null server");
    Server *s = reinterpret_cast<Server *>(server);
    std::unique_lock<std::mutex> lock(s->mu);
    bool ok = s->cv.wait_for(lock, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                             [s] { return s->pending == 0; });
    if (!ok) return set_error(GXY_ERR_TIMEOUT, "requests still running after the timeout");
    return GXY_OK;
}

int gxy_server_take(gxy_server server, int64_t id, float *rgba, double *latency_s, int64_t *rays) {
    if (!server) return set_error(GXY_ERR_INVALID, "null server");
    Server *s = reinterpret_cast<Server *>(server);
    SReq r;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        auto it = s->reqs.find(id);
        if (it == s->reqs.end()) return set_error(GXY_ERR_INVALID, "unknown request");
        if (it->second.state < R_DONE) return set_error(GXY_ERR_INVALID, "request not finished");
        r = it->second;
        s->reqs.erase(it);
        s->fb_used -= r.fb_bytes;
    }
    if (latency_s) *latency_s = r.t_done - r.arrival;
    if (rays) *rays = r.rays;
    int rc = GXY_OK;
    if (r.fb) {
        if (rgba && r.state == R_DONE)
            if (cudaMemcpyAsync(rgba, r.fb, r.fb_bytes, cudaMemcpyDeviceToHost, s->io) != cudaSuccess)
                rc = set_error(GXY_ERR_CUDA, "framebuffer copy failed");
        cudaFreeAsync(r.fb, s->io);
        cudaStreamSynchronize(s->io);
    }
    if (r.state == R_FAILED)
        return set_error(r.error ? r.error : GXY_ERR_CUDA, "request failed: " + r.message);
    return rc;
}

}  // extern "C"
