// cm_server.cpp -- request server over the engine handles: continuous
// batching of MDDF jobs on one device.
//
// A request is one system (cm_system_desc) with its frames in host or device
// memory (the caller keeps them valid until the request is done).
// Requests wait in arrival order until the server admits them: a request is
// admitted when fewer than max_active requests are on the device and its
// handle's memory fits in what is left of the server's HBM budget (the handle
// is created with that remainder as its own budget, so a request that does not
// fit fails its first allocation and goes back to the queue; smaller requests
// behind it may be admitted first).  Each admitted request owns a handle --
// coordinates, cell lists and int64 accumulators resident on the device -- and
// its own stream, so the work of all admitted requests overlaps on the GPU.
// The scheduler thread gives each admitted request a turn of frames_per_turn
// frames in round-robin order, and reads a request's counts back as soon as
// its last frame has finished, freeing its device memory for the next ones.
// Latency is measured on the host from submit to the read-back of the counts.
//
// Replaces (ComplexMixtures.jl): nothing -- the reference runs one mddf call
// at a time; each request's result is the one mddf (src/mddf.jl:227-347)
// would give for its trajectory and options.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/cmgpu.h"

namespace {

using Clock = std::chrono::steady_clock;

thread_local std::string t_server_error;

struct Request {
    int64_t id = 0;
    cm_system_desc desc{};
    std::vector<int64_t> gs_off, gv_off;
    std::vector<int32_t> gs_idx, gv_idx;
    // frames: coordinates referenced, the rest copied
    cm_frames frames{};
    std::vector<double> cells, weights;
    std::vector<int64_t> ids;
    int64_t next = 0;           // next frame to submit
    cm_handle *h = nullptr;
    cudaEvent_t done_ev = nullptr;
    int state = CM_REQ_QUEUED;
    int status = CM_OK;
    std::string error;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int64_t device_bytes = 0;
    int64_t reserved_bytes = 0;
    // results (read back at completion)
    int64_t nbins = 0, Gs = 0, Gv = 0;
    std::vector<int64_t> raw;   // md, md_r, rdf, rdf_r, gs, gs_r, gv, gv_r (half units)
    std::vector<double> wsum;   // the same, weighted
    double volume_total = 0, weight_total = 0;
    int64_t frames_done = 0;
    bool raw_valid = false;
};

}  // namespace

struct cm_server {
    cm_server_desc d{};
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<int64_t> queue;
    std::vector<int64_t> active;
    std::map<int64_t, std::unique_ptr<Request>> reqs;
    int64_t next_id = 1;
    int64_t used_bytes = 0;
    bool stop = false;
    std::thread worker;
    std::string err;
};

namespace {

double now_s(const cm_server *s) { return std::chrono::duration<double>(Clock::now() - s->t0).count(); }

// Copy of a request's description with its own group tables.
void own_desc(Request &r, const cm_system_desc *d) {
    r.desc = *d;
    const int64_t aps = d->solute_natomspermol, Nv = (int64_t)d->solvent_nmols * d->solvent_natomspermol;
    if (d->solute_group_offsets) {
        r.gs_off.assign(d->solute_group_offsets, d->solute_group_offsets + aps + 1);
        r.gs_idx.assign(d->solute_groups, d->solute_groups + r.gs_off[aps]);
        if (r.gs_idx.empty()) r.gs_idx.push_back(0);
        r.desc.solute_group_offsets = r.gs_off.data();
        r.desc.solute_groups = r.gs_idx.data();
    }
    if (d->solvent_group_offsets) {
        r.gv_off.assign(d->solvent_group_offsets, d->solvent_group_offsets + Nv + 1);
        r.gv_idx.assign(d->solvent_groups, d->solvent_groups + r.gv_off[Nv]);
        if (r.gv_idx.empty()) r.gv_idx.push_back(0);
        r.desc.solvent_group_offsets = r.gv_off.data();
        r.desc.solvent_groups = r.gv_idx.data();
    }
    r.nbins = d->nbins;
    r.Gs = d->solute_group_offsets ? d->solute_ngroups : d->solute_natomspermol;
    r.Gv = d->solvent_group_offsets ? d->solvent_ngroups : d->solvent_natomspermol;
}

void fail(Request &r, int st, const std::string &msg) {
    r.state = CM_REQ_FAILED;
    r.status = st;
    r.error = msg;
}

void release_device(cm_server *s, Request &r) {
    if (r.done_ev) cudaEventDestroy(r.done_ev);
    r.done_ev = nullptr;
    if (r.h) cm_destroy(r.h);
    r.h = nullptr;
    s->used_bytes -= r.reserved_bytes;
    r.reserved_bytes = 0;
}

// Frames [r.next, r.next + n) of a request.
int submit_turn(Request &r, int64_t n) {
    cm_frames f = r.frames;
    const int64_t k = r.next;
    const int64_t Ns = (int64_t)r.desc.solute_nmols * r.desc.solute_natomspermol;
    const int64_t Nv = (int64_t)r.desc.solvent_nmols * r.desc.solvent_natomspermol;
    const int64_t elem = f.coord_type == CM_COORD_F32 ? 4 : 8;
    const int64_t ss = f.solute_frame_stride > 0 ? f.solute_frame_stride : Ns * 3;
    const int64_t vs = f.solvent_frame_stride > 0 ? f.solvent_frame_stride : Nv * 3;
    f.nframes = (int32_t)n;
    f.solute_xyz = (const char *)r.frames.solute_xyz + k * ss * elem;
    f.solvent_xyz = r.frames.solvent_xyz ? (const char *)r.frames.solvent_xyz + k * vs * elem : nullptr;
    f.cells = r.cells.data() + 9 * k;
    f.weights = r.weights.empty() ? nullptr : r.weights.data() + k;
    f.frame_ids = r.ids.data() + k;
    const int st = cm_submit_frames(r.h, &f);
    if (st == CM_OK) r.next += n;
    return st;
}

// Try to put a queued request on the device; false if it does not fit now.
bool admit(cm_server *s, Request &r) {
    const int64_t left = s->d.hbm_budget_bytes > 0 ? s->d.hbm_budget_bytes - s->used_bytes : 0;
    if (s->d.hbm_budget_bytes > 0 && left <= 0) return false;
    cm_system_desc d = r.desc;
    d.device = s->d.device;
    d.hbm_budget_bytes = left;
    d.max_frames_per_batch = std::max(1, s->d.frames_per_turn);
    cm_handle *h = nullptr;
    int st = cm_create(&d, &h);
    if (st == CM_ENOMEM) return false;
    if (st != CM_OK) {
        fail(r, st, cm_last_error(nullptr));
        r.t_done = now_s(s);
        return true;
    }
    r.h = h;
    // the first turn allocates the handle's working set
    st = submit_turn(r, std::min<int64_t>(std::max(1, s->d.frames_per_turn), r.frames.nframes));
    if (st == CM_ENOMEM) {
        cm_destroy(h);
        r.h = nullptr;
        r.next = 0;
        return false;
    }
    r.device_bytes = cm_device_bytes(h);
    // reserve a quarter more for cell arrays that later frames may need
    r.reserved_bytes = s->d.hbm_budget_bytes > 0 ? std::min<int64_t>(left, r.device_bytes + r.device_bytes / 4)
                                                  : r.device_bytes;
    s->used_bytes += r.reserved_bytes;
    r.t_admit = now_s(s);
    r.state = CM_REQ_RUNNING;
    if (st != CM_OK) {
        fail(r, st, cm_last_error(h));
        release_device(s, r);
        r.t_done = now_s(s);
    } else if (r.next == r.frames.nframes) {
        cudaEventCreateWithFlags(&r.done_ev, cudaEventDisableTiming);
        cudaEventRecord(r.done_ev, (cudaStream_t)cm_stream(h));
    }
    return true;
}

// Read the counts of a request whose last frame has finished.
void finish(cm_server *s, Request &r) {
    const int64_t nb = r.nbins;
    const int64_t n = nb * (4 + 2 * r.Gs + 2 * r.Gv);
    r.raw.assign(n, 0);
    r.wsum.assign(n, 0.0);
    int64_t *p = r.raw.data();
    cm_raw_counts rc{p, p + nb, p + 2 * nb, p + 3 * nb, p + 4 * nb, p + 4 * nb + r.Gs * nb, p + 4 * nb + 2 * r.Gs * nb,
                     p + 4 * nb + 2 * r.Gs * nb + r.Gv * nb};
    double *w = r.wsum.data();
    cm_counts cc{w, w + nb, w + 2 * nb, w + 3 * nb, w + 4 * nb, w + 4 * nb + r.Gs * nb, w + 4 * nb + 2 * r.Gs * nb,
                 w + 4 * nb + 2 * r.Gs * nb + r.Gv * nb, 0.0, 0.0, 0};
    int st = cm_read_counts(r.h, &cc);
    if (st == CM_OK) {
        r.volume_total = cc.volume_total;
        r.weight_total = cc.weight_total;
        r.frames_done = cc.frames;
        const int st2 = cm_read_raw_counts(r.h, &rc);
        r.raw_valid = st2 == CM_OK;
        r.state = CM_REQ_DONE;
    } else {
        fail(r, st, cm_last_error(r.h));
    }
    release_device(s, r);
    r.t_done = now_s(s);
}

void scheduler(cm_server *s) {
    cudaSetDevice(s->d.device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        if (s->stop) break;
        // admission: first-fit over the queue in arrival order
        const int max_active = s->d.max_active > 0 ? s->d.max_active : 1 << 30;
        for (auto it = s->queue.begin(); it != s->queue.end() && (int)s->active.size() < max_active;) {
            Request &r = *s->reqs[*it];
            if (r.state == CM_REQ_CANCELLED) {
                it = s->queue.erase(it);
                continue;
            }
            if (admit(s, r)) {
                if (r.state == CM_REQ_RUNNING) s->active.push_back(r.id);
                else s->cv_done.notify_all();
                it = s->queue.erase(it);
            } else {
                ++it;
            }
        }
        if (s->active.empty()) {
            if (s->queue.empty()) {
                s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty(); });
                continue;
            }
            // every queued request was tried on an idle device and none fits:
            // the head request cannot run at all
            Request &r = *s->reqs[s->queue.front()];
            fail(r, CM_ENOMEM, "request does not fit in device memory or in the server's HBM budget");
            r.t_done = now_s(s);
            s->queue.pop_front();
            s->cv_done.notify_all();
            continue;
        }
        // one turn per active request, round robin
        bool progressed = false;
        for (size_t i = 0; i < s->active.size(); ++i) {
            Request &r = *s->reqs[s->active[i]];
            if (r.state != CM_REQ_RUNNING) continue;
            if (r.next < r.frames.nframes) {
                const int64_t n = std::min<int64_t>(std::max(1, s->d.frames_per_turn), r.frames.nframes - r.next);
                // the request stays active (and its handle alive) while the
                // lock is released: only this thread removes active requests
                lk.unlock();
                const int st = submit_turn(r, n);
                lk.lock();
                if (st != CM_OK) {
                    fail(r, st, cm_last_error(r.h));
                    release_device(s, r);
                    r.t_done = now_s(s);
                    continue;
                }
                progressed = true;
                if (r.next == r.frames.nframes) {
                    cudaEventCreateWithFlags(&r.done_ev, cudaEventDisableTiming);
                    cudaEventRecord(r.done_ev, (cudaStream_t)cm_stream(r.h));
                }
            }
        }
        // completions
        for (size_t i = 0; i < s->active.size();) {
            Request &r = *s->reqs[s->active[i]];
            bool remove = r.state != CM_REQ_RUNNING;
            if (!remove && r.next == r.frames.nframes && cudaEventQuery(r.done_ev) == cudaSuccess) {
                finish(s, r);
                remove = true;
            }
            if (r.state == CM_REQ_CANCELLED && r.h) release_device(s, r);
            if (remove) {
                s->active.erase(s->active.begin() + i);
                s->cv_done.notify_all();
                progressed = true;
            } else {
                ++i;
            }
        }
        if (!progressed) {
            // everything submitted: let the GPU work without spinning the host
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(200));
            lk.lock();
        }
    }
    for (int64_t id : s->active) {
        Request &r = *s->reqs[id];
        if (r.h) release_device(s, r);
    }
}

Request *find(cm_server *s, int64_t id) {
    auto it = s->reqs.find(id);
    return it == s->reqs.end() ? nullptr : it->second.get();
}

int server_fail(cm_server *s, int code, const std::string &msg) {
    if (s) s->err = msg;
    else t_server_error = msg;
    return code;
}

void info_of(const Request &r, cm_request_info *out) {
    memset(out, 0, sizeof(*out));
    out->state = r.state;
    out->status = r.status;
    out->t_submit = r.t_submit;
    out->t_admit = r.t_admit;
    out->t_done = r.t_done;
    out->frames_submitted = r.next;
    out->device_bytes = r.device_bytes;
}

}  // namespace

extern "C" {

int cm_server_create(const cm_server_desc *desc, cm_server **out) {
    if (!out || !desc) return server_fail(nullptr, CM_EINVAL, "NULL argument");
    *out = nullptr;
    if (desc->frames_per_turn < 0 || desc->max_active < 0 || desc->hbm_budget_bytes < 0)
        return server_fail(nullptr, CM_EINVAL, "negative server parameter");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || desc->device < 0 || desc->device >= ndev)
        return server_fail(nullptr, CM_EDEVICE, "no such CUDA device");
    cm_server *s = new cm_server();
    s->d = *desc;
    if (s->d.frames_per_turn == 0) s->d.frames_per_turn = 32;
    s->t0 = Clock::now();
    s->worker = std::thread(scheduler, s);
    *out = s;
    return CM_OK;
}

int cm_server_submit(cm_server *s, const cm_system_desc *desc, const cm_frames *frames, int64_t *request_id) {
    if (!s || !desc || !frames || !request_id) return server_fail(s, CM_EINVAL, "NULL argument");
    if (frames->memory != CM_MEM_HOST && frames->memory != CM_MEM_DEVICE)
        return server_fail(s, CM_EINVAL, "unknown memory kind");
    if (frames->coord_type != CM_COORD_F32 && frames->coord_type != CM_COORD_F64)
        return server_fail(s, CM_EINVAL, "server requests take FP32 or FP64 coordinates");
    if (frames->nframes < 1 || !frames->solute_xyz || !frames->cells || !frames->frame_ids)
        return server_fail(s, CM_EINVAL, "a request needs at least one frame with coordinates, cells and frame ids");
    if (!desc->autocorrelation && !frames->solvent_xyz) return server_fail(s, CM_EINVAL, "solvent_xyz is required");
    auto r = std::make_unique<Request>();
    own_desc(*r, desc);
    r->frames = *frames;
    const int64_t n = frames->nframes;
    r->cells.assign(frames->cells, frames->cells + 9 * n);
    if (frames->weights) r->weights.assign(frames->weights, frames->weights + n);
    r->ids.assign(frames->frame_ids, frames->frame_ids + n);
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    r->t_submit = now_s(s);
    *request_id = r->id;
    s->queue.push_back(r->id);
    s->reqs[r->id] = std::move(r);
    s->cv_work.notify_all();
    return CM_OK;
}

int cm_server_poll(cm_server *s, int64_t id, cm_request_info *out) {
    if (!s || !out) return server_fail(s, CM_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    Request *r = find(s, id);
    if (!r) return server_fail(s, CM_EINVAL, "unknown request id");
    info_of(*r, out);
    return CM_OK;
}

int cm_server_wait(cm_server *s, int64_t id, double timeout_s, cm_request_info *out) {
    if (!s) return server_fail(s, CM_EINVAL, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    Request *r = find(s, id);
    if (!r) return server_fail(s, CM_EINVAL, "unknown request id");
    auto finished = [&] { return r->state == CM_REQ_DONE || r->state == CM_REQ_FAILED || r->state == CM_REQ_CANCELLED; };
    if (timeout_s < 0) s->cv_done.wait(lk, finished);
    else s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished);
    if (out) info_of(*r, out);
    return finished() ? CM_OK : server_fail(s, CM_ESTATE, "request still running at the timeout");
}

int cm_server_read_counts(cm_server *s, int64_t id, cm_counts *out) {
    if (!s || !out) return server_fail(s, CM_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    Request *r = find(s, id);
    if (!r) return server_fail(s, CM_EINVAL, "unknown request id");
    if (r->state != CM_REQ_DONE)
        return server_fail(s, r->state == CM_REQ_FAILED ? r->status : CM_ESTATE,
                           r->state == CM_REQ_FAILED ? r->error : "request not finished");
    const int64_t nb = r->nbins;
    const double *w = r->wsum.data();
    auto put = [&](double *dst, const double *src, int64_t n) {
        if (dst) memcpy(dst, src, n * 8);
    };
    put(out->md_count, w, nb);
    put(out->md_count_random, w + nb, nb);
    put(out->rdf_count, w + 2 * nb, nb);
    put(out->rdf_count_random, w + 3 * nb, nb);
    put(out->solute_group_count, w + 4 * nb, r->Gs * nb);
    put(out->solute_group_count_random, w + 4 * nb + r->Gs * nb, r->Gs * nb);
    put(out->solvent_group_count, w + 4 * nb + 2 * r->Gs * nb, r->Gv * nb);
    put(out->solvent_group_count_random, w + 4 * nb + 2 * r->Gs * nb + r->Gv * nb, r->Gv * nb);
    out->volume_total = r->volume_total;
    out->weight_total = r->weight_total;
    out->frames = r->frames_done;
    return CM_OK;
}

int cm_server_read_raw_counts(cm_server *s, int64_t id, cm_raw_counts *out) {
    if (!s || !out) return server_fail(s, CM_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    Request *r = find(s, id);
    if (!r) return server_fail(s, CM_EINVAL, "unknown request id");
    if (r->state != CM_REQ_DONE)
        return server_fail(s, r->state == CM_REQ_FAILED ? r->status : CM_ESTATE,
                           r->state == CM_REQ_FAILED ? r->error : "request not finished");
    if (!r->raw_valid) return server_fail(s, CM_ESTATE, "raw counts are defined only while all frames carry one weight");
    const int64_t nb = r->nbins;
    const int64_t *p = r->raw.data();
    auto put = [&](int64_t *dst, const int64_t *src, int64_t n) {
        if (dst) memcpy(dst, src, n * 8);
    };
    put(out->md, p, nb);
    put(out->md_random, p + nb, nb);
    put(out->rdf, p + 2 * nb, nb);
    put(out->rdf_random, p + 3 * nb, nb);
    put(out->solute_group, p + 4 * nb, r->Gs * nb);
    put(out->solute_group_random, p + 4 * nb + r->Gs * nb, r->Gs * nb);
    put(out->solvent_group, p + 4 * nb + 2 * r->Gs * nb, r->Gv * nb);
    put(out->solvent_group_random, p + 4 * nb + 2 * r->Gs * nb + r->Gv * nb, r->Gv * nb);
    return CM_OK;
}

int cm_server_cancel(cm_server *s, int64_t id) {
    if (!s) return server_fail(s, CM_EINVAL, "NULL server");
    std::lock_guard<std::mutex> lk(s->mu);
    Request *r = find(s, id);
    if (!r) return server_fail(s, CM_EINVAL, "unknown request id");
    if (r->state == CM_REQ_QUEUED || r->state == CM_REQ_RUNNING) {
        r->state = CM_REQ_CANCELLED;
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
    return CM_OK;
}

int cm_server_release(cm_server *s, int64_t id) {
    if (!s) return server_fail(s, CM_EINVAL, "NULL server");
    std::lock_guard<std::mutex> lk(s->mu);
    Request *r = find(s, id);
    if (!r) return server_fail(s, CM_EINVAL, "unknown request id");
    if (r->state == CM_REQ_QUEUED || r->state == CM_REQ_RUNNING)
        return server_fail(s, CM_ESTATE, "request still queued or running (cancel it first)");
    if (r->h) return server_fail(s, CM_ESTATE, "request still holds device state");
    s->reqs.erase(id);
    return CM_OK;
}

int cm_server_destroy(cm_server *s) {
    if (!s) return CM_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    delete s;
    return CM_OK;
}

const char *cm_server_last_error(const cm_server *s) { return s ? s->err.c_str() : t_server_error.c_str(); }

}  // extern "C"
