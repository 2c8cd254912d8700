// server.cu -- the served form: a request loop over voxelize-and-gather jobs.
//
// Jobs (point set + path parameters) are queued by gbvdb_server_submit and run
// by worker threads, each with its own CUDA stream and its own reusable grid,
// so that jobs that arrive while others are on the GPU overlap there (their
// kernels run concurrently, and each job's few host round trips block only its
// own worker).  A job either builds a fresh grid (freed for the next job) or
// updates a resident grid by id, whose topology, pools and atlas stay on the
// device between jobs (later jobs on it take the incremental rebuild path).
// Admission: a job starts only while the device bytes held by all grids plus
// the job's estimate stay within the memory cap (at least one job always
// runs), and jobs on one resident grid run in submission order.
//
// Each job is the reference's per-frame call sequence on a VolumeGVDB
// (source/gFluidSurface/main_fluid_surface.cpp:325-356): SetPoints,
// RebuildTopology, UpdateAtlas, InsertPointsSubcell, GatherDensity or
// GatherLevelSet, UpdateApron, followed by the FP64 channel checksum.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "gbvdb.h"

extern "C" size_t gbvdb_internal_device_bytes(gbvdb_grid g);  // grid.cu (not exported)

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct JobRec {
    gbvdb_job desc;
    int64_t ticket = 0;
    size_t estimate = 0;
    bool done = false;
    gbvdb_job_result res{};
};

struct Resident {
    gbvdb_grid g = nullptr;
    bool busy = false;
    int dtype = -1;
    int levs = 0;
    int log2dim[8] = {0};
    void* dpts = nullptr;  // device copy of the grid's current points
    size_t dpts_cap = 0;
};

// a reusable grid + point buffer owned by one worker
struct Slot {
    gbvdb_grid g = nullptr;
    int dtype = -1;
    void* dpts = nullptr;
    size_t dpts_cap = 0;
};

size_t job_estimate(const gbvdb_job& j) {
    // points (input copy, binned records, per-point scratch) + a brick estimate
    // (one 16^3 brick per 64 points, at least 64) x (interior + apron) x element size
    size_t es = j.dtype == GBVDB_T_FLOAT ? 4 : 2;
    size_t n = (size_t)(j.n > 0 ? j.n : 0);
    size_t bricks = n / 64 + 64;
    return n * 48 + bricks * (4096 + 1744) * es + ((size_t)64 << 20);
}

}  // namespace

struct gbvdb_server_s {
    int device = 0;
    size_t cap = 0;
    std::vector<std::thread> workers;
    std::vector<cudaStream_t> streams;  // one per worker, alive until every grid is destroyed
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<JobRec*> queue;
    std::map<int64_t, JobRec*> jobs;
    std::map<int32_t, Resident> resident;
    int64_t next_ticket = 1;
    size_t held = 0;      // device bytes of the grids, as of their last job
    size_t inflight = 0;  // estimates of running jobs
    int running = 0;
    bool stop = false;
    std::vector<size_t> slot_bytes;
    double t0 = 0;
    int64_t completed = 0;
    double busy_ms = 0;
    std::string err;

    bool grid_busy(int32_t rid) {
        if (rid < 0) return false;
        auto it = resident.find(rid);
        return it != resident.end() && it->second.busy;
    }
    bool fits(const JobRec* j) const { return running == 0 || held + inflight + j->estimate <= cap; }

    // The next runnable job in submission order.  A job whose resident grid is
    // busy waits (and so do the later jobs of that grid) while later jobs may
    // pass it; a job that does not fit under the memory cap stops the scan, so
    // admission by memory stays first come, first served.
    JobRec* take() {
        for (auto it = queue.begin(); it != queue.end(); ++it) {
            JobRec* j = *it;
            if (grid_busy(j->desc.resident_id)) continue;
            if (!fits(j)) return nullptr;
            queue.erase(it);
            return j;
        }
        return nullptr;
    }

    void worker(int wi) {
        cudaSetDevice(device);
        cudaStream_t st = streams[(size_t)wi];
        Slot slot;
        while (true) {
            JobRec* j = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] {
                    if (stop && queue.empty()) return true;
                    j = take();
                    return j != nullptr;
                });
                if (!j) break;
                running++;
                inflight += j->estimate;
                if (j->desc.resident_id >= 0) {
                    Resident& r = resident[j->desc.resident_id];
                    r.busy = true;
                }
            }
            j->res.t_start_ms = now_ms() - t0;
            Resident* rp = nullptr;
            if (j->desc.resident_id >= 0) {
                std::lock_guard<std::mutex> lk(mu);
                rp = &resident[j->desc.resident_id];
            }
            gbvdb_status stt = run(*j, st, slot, rp);
            cudaStreamSynchronize(st);
            j->res.t_end_ms = now_ms() - t0;
            j->res.status = (int32_t)stt;
            {
                std::lock_guard<std::mutex> lk(mu);
                running--;
                inflight -= j->estimate;
                if (rp) rp->busy = false;
                // held bytes: this worker's slot + every resident grid
                slot_bytes[(size_t)wi] = slot.g ? gbvdb_internal_device_bytes(slot.g) : 0;
                size_t h = 0;
                for (size_t b : slot_bytes) h += b;
                for (auto& kv : resident) h += gbvdb_internal_device_bytes(kv.second.g) + kv.second.dpts_cap;
                held = h;
                j->done = true;
                completed++;
                busy_ms += j->res.t_end_ms - j->res.t_start_ms;
            }
            cv_done.notify_all();
            cv_work.notify_all();
        }
        if (slot.g) gbvdb_destroy(slot.g);
        if (slot.dpts) cudaFreeAsync(slot.dpts, st);
        cudaStreamSynchronize(st);
    }

    gbvdb_status setup_grid(gbvdb_grid& g, int& have_dtype, const gbvdb_job& d, cudaStream_t st) {
        gbvdb_status s;
        if (!g) {
            if ((s = gbvdb_create(device, &g)) != GBVDB_OK) return s;
            have_dtype = -1;
        }
        if ((s = gbvdb_set_stream(g, st)) != GBVDB_OK) return s;
        if ((s = gbvdb_configure(g, d.levs, d.log2dim_leaf_first)) != GBVDB_OK) return s;
        if (have_dtype != d.dtype) {
            if ((s = gbvdb_add_channel(g, 0, d.dtype, 1, 0, 0, 0)) != GBVDB_OK) return s;
            have_dtype = d.dtype;
        }
        return GBVDB_OK;
    }

    gbvdb_status run(JobRec& j, cudaStream_t st, Slot& slot, Resident* rp) {
        const gbvdb_job& d = j.desc;
        gbvdb_status s;
        gbvdb_grid g;
        void** dpts;
        size_t* dcap;
        if (rp) {
            bool same = rp->g && rp->levs == d.levs && rp->dtype == d.dtype;
            for (int l = 0; same && l < d.levs; l++) same = rp->log2dim[l] == d.log2dim_leaf_first[l];
            if (!same) {
                if ((s = setup_grid(rp->g, rp->dtype, d, st)) != GBVDB_OK) return s;
                rp->levs = d.levs;
                for (int l = 0; l < d.levs; l++) rp->log2dim[l] = d.log2dim_leaf_first[l];
            } else if ((s = gbvdb_set_stream(rp->g, st)) != GBVDB_OK) {
                return s;
            }
            g = rp->g;
            dpts = &rp->dpts;
            dcap = &rp->dpts_cap;
        } else {
            if ((s = setup_grid(slot.g, slot.dtype, d, st)) != GBVDB_OK) return s;
            g = slot.g;
            dpts = &slot.dpts;
            dcap = &slot.dpts_cap;
        }
        const void* src = d.points;
        int stride = d.stride ? d.stride : 12;
        if (!d.points_on_device && d.n > 0) {
            size_t bytes = (size_t)d.n * (size_t)stride;
            if (*dcap < bytes) {
                if (*dpts) cudaFreeAsync(*dpts, st);
                *dpts = nullptr;
                *dcap = 0;
                if (cudaMallocAsync(dpts, bytes, st) != cudaSuccess) {
                    cudaGetLastError();
                    return GBVDB_OUT_OF_MEMORY;
                }
                *dcap = bytes;
            }
            if (cudaMemcpyAsync(*dpts, d.points, bytes, cudaMemcpyHostToDevice, st) != cudaSuccess) return GBVDB_CUDA_ERROR;
            src = *dpts;
        }
        if ((s = gbvdb_set_points(g, src, d.n, 0, stride, nullptr, 0, 0, nullptr, 0, 0)) != GBVDB_OK) return s;
        s = gbvdb_rebuild_topology(g, d.n, d.radius, d.orig);
        if (s == GBVDB_DEPTH_UNSUPPORTED || s == GBVDB_NOOP) return s;
        if (s != GBVDB_OK) return s;
        if ((s = gbvdb_update_atlas(g)) != GBVDB_OK) return s;
        int64_t len = 0;
        s = gbvdb_insert_points_subcell(g, 4, d.n, d.insert_radius, d.orig, &len);
        if (s != GBVDB_OK && s != GBVDB_NOOP) return s;
        if (d.mode == 0)
            s = gbvdb_gather_density(g, 4, d.n, d.gather_radius, d.orig, len, 0, -1, 0);
        else
            s = gbvdb_gather_levelset(g, 4, d.n, d.gather_radius, d.orig, len, 0, -1, 0);
        if (s != GBVDB_OK && s != GBVDB_NOOP) return s;
        s = gbvdb_update_apron(g, 0, d.boundval);
        if (s != GBVDB_OK && s != GBVDB_NOOP) return s;
        if ((s = gbvdb_checksum(g, 0, &j.res.checksum)) != GBVDB_OK) return s;
        int64_t st4[4];
        gbvdb_get_stats(g, st4);
        j.res.sc_len = st4[2];
        j.res.bricks = st4[3];
        return GBVDB_OK;
    }
};

extern "C" {

gbvdb_status gbvdb_server_create(int device, int workers, int64_t mem_cap_bytes, gbvdb_server* out) {
    if (!out || workers < 1 || workers > 64 || mem_cap_bytes <= 0) return GBVDB_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return GBVDB_CUDA_ERROR;
    }
    gbvdb_server s = new (std::nothrow) gbvdb_server_s();
    if (!s) return GBVDB_OUT_OF_MEMORY;
    s->device = device;
    s->cap = (size_t)mem_cap_bytes;
    s->t0 = now_ms();
    s->slot_bytes.assign((size_t)workers, 0);
    cudaSetDevice(device);
    for (int i = 0; i < workers; i++) {
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
            for (cudaStream_t x : s->streams) cudaStreamDestroy(x);
            delete s;
            return GBVDB_CUDA_ERROR;
        }
        s->streams.push_back(st);
    }
    for (int i = 0; i < workers; i++) s->workers.emplace_back([s, i] { s->worker(i); });
    *out = s;
    return GBVDB_OK;
}

gbvdb_status gbvdb_server_submit(gbvdb_server s, const gbvdb_job* job, int64_t* ticket) {
    if (!s || !job || !ticket) return GBVDB_INVALID_ARG;
    if (job->n < 0 || (job->n > 0 && !job->points) || job->levs < 2 || job->levs > 8) return GBVDB_INVALID_ARG;
    if (job->stride != 0 && job->stride < 12) return GBVDB_INVALID_ARG;
    JobRec* j = new (std::nothrow) JobRec();
    if (!j) return GBVDB_OUT_OF_MEMORY;
    j->desc = *job;
    j->estimate = job_estimate(*job);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            delete j;
            return GBVDB_INVALID_ARG;
        }
        j->ticket = s->next_ticket++;
        j->res.t_submit_ms = now_ms() - s->t0;
        s->jobs[j->ticket] = j;
        s->queue.push_back(j);
        *ticket = j->ticket;
    }
    s->cv_work.notify_one();
    return GBVDB_OK;
}

gbvdb_status gbvdb_server_wait(gbvdb_server s, int64_t ticket, gbvdb_job_result* out) {
    if (!s || !out) return GBVDB_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return GBVDB_INVALID_ARG;
    JobRec* j = it->second;
    s->cv_done.wait(lk, [&] { return j->done; });
    *out = j->res;
    s->jobs.erase(it);
    delete j;
    return GBVDB_OK;
}

gbvdb_status gbvdb_server_poll(gbvdb_server s, int64_t ticket, int* done) {
    if (!s || !done) return GBVDB_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return GBVDB_INVALID_ARG;
    *done = it->second->done ? 1 : 0;
    return GBVDB_OK;
}

gbvdb_status gbvdb_server_resident(gbvdb_server s, int32_t resident_id, gbvdb_grid* out) {
    if (!s || !out) return GBVDB_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->resident.find(resident_id);
    if (it == s->resident.end() || !it->second.g || it->second.busy) return GBVDB_INVALID_ARG;
    *out = it->second.g;
    return GBVDB_OK;
}

gbvdb_status gbvdb_server_release(gbvdb_server s, int32_t resident_id) {
    if (!s) return GBVDB_INVALID_ARG;
    Resident r;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->resident.find(resident_id);
        if (it == s->resident.end() || it->second.busy) return GBVDB_INVALID_ARG;
        for (JobRec* j : s->queue)
            if (j->desc.resident_id == resident_id) return GBVDB_INVALID_ARG;  // jobs still queued for it
        r = it->second;
        s->resident.erase(it);
    }
    cudaSetDevice(s->device);
    if (r.g) gbvdb_destroy(r.g);
    if (r.dpts) cudaFree(r.dpts);
    return GBVDB_OK;
}

gbvdb_status gbvdb_server_stats(gbvdb_server s, int64_t* out6) {
    if (!s || !out6) return GBVDB_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    out6[0] = (int64_t)s->queue.size();
    out6[1] = s->running;
    out6[2] = s->completed;
    out6[3] = (int64_t)s->held;
    out6[4] = (int64_t)s->cap;
    out6[5] = (int64_t)s->resident.size();
    return GBVDB_OK;
}

gbvdb_status gbvdb_server_destroy(gbvdb_server s) {
    if (!s) return GBVDB_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    cudaSetDevice(s->device);
    for (auto& kv : s->resident) {
        if (kv.second.g) gbvdb_destroy(kv.second.g);
        if (kv.second.dpts) cudaFree(kv.second.dpts);
    }
    for (auto& kv : s->jobs) delete kv.second;
    for (cudaStream_t st : s->streams) cudaStreamDestroy(st);
    delete s;
    return GBVDB_OK;
}

}  // extern "C"
