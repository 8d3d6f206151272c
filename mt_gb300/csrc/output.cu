// output.cu - stride-step outputs without stalling the step loop: DCD frames
// of the coordinates and angles of every trajectory and the per-trajectory
// energy lines, through pinned double buffers and a host writer thread.
//
// The reference downloads r synchronously at every stride step
// (src/compute_cuda.cu:1177) and writes each trajectory's frame to two DCD
// files (saveCoordDCD, src/preparator.cpp:582-602, frames as dcdWriteFrame,
// src/dcdio.cpp:179-203; headers as dcdWriteHeader, :98-154) and prints the
// energy totals (OutputAllEnergies, src/updater.cpp:3-43).  Here a frame
// request converts the state on the engine's stream into a slot's device
// buffer, a copy stream moves it to the slot's pinned host buffer, and the
// writer thread turns it into the same bytes in the same files once the copy
// event has completed; the step loop continues meanwhile.  The DCD layout is
// the reference's (no unit cell): header
//   84 "CORD" nfile npriv nsavc npriv-nsavc 0x5 delta 0(hasUC) 0x8 24 84
//   164 2 remark1[80] remark2[80] 164 4 N 4
// and per frame  4N X[N] 4N 4N Y[N] 4N 4N Z[N] 4N  (int32 / float32), with
// (x, y, z) in the xyz file and (fi, psi, theta) in the angle file.
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "mtg_engine.cuh"

using namespace mtg;

struct mtg_output {
    static constexpr int kSlots = 2;
    int device = 0, nb = 0, nt = 0;
    std::vector<int> off;
    std::vector<std::string> xyz, ang;
    cudaStream_t copy = nullptr;
    float *d_stage[kSlots] = {nullptr, nullptr};
    double *d_en[kSlots] = {nullptr, nullptr};
    float *h_coords[kSlots] = {nullptr, nullptr};
    double *h_en[kSlots] = {nullptr, nullptr};
    cudaEvent_t converted[kSlots] = {nullptr, nullptr}, copied[kSlots] = {nullptr, nullptr};
    int *d_ignored_err = nullptr;   // non-finite totals are printed, not raised (as the reference)
    struct Job {
        int slot;
        long long step;
        bool frame, energies;
    };
    std::mutex m;
    std::condition_variable cv;
    std::deque<Job> jobs;
    bool busy[kSlots] = {false, false};
    bool stop = false;
    int error = 0;           // first failure of the writer thread
    std::string error_msg;
    FILE *energy_out = stdout;
    std::thread writer;
    long long frames_written = 0;
};

namespace {

void put_i32(FILE *f, int v, bool &ok) { ok = ok && std::fwrite(&v, 4, 1, f) == 1; }

bool write_header(const char *path, int N, int nfile, int npriv, int nsavc, float delta, const char *remark2) {
    FILE *f = std::fopen(path, "w");
    if (!f) return false;
    bool ok = true;
    put_i32(f, 84, ok);
    ok = ok && std::fwrite("CORD", 4, 1, f) == 1;
    put_i32(f, nfile, ok);
    put_i32(f, npriv, ok);
    put_i32(f, nsavc, ok);
    put_i32(f, npriv - nsavc, ok);
    for (int i = 0; i < 5; i++) put_i32(f, 0, ok);
    ok = ok && std::fwrite(&delta, 4, 1, f) == 1;
    put_i32(f, 0, ok);   // no unit cell
    for (int i = 0; i < 8; i++) put_i32(f, 0, ok);
    put_i32(f, 24, ok);
    put_i32(f, 84, ok);
    put_i32(f, 164, ok);
    put_i32(f, 2, ok);
    char title[80];
    std::memset(title, 0, sizeof title);
    std::strncpy(title, "REMARKS CREATED BY dcdio.c", sizeof title - 1);
    ok = ok && std::fwrite(title, 80, 1, f) == 1;
    std::memset(title, 0, sizeof title);
    std::strncpy(title, remark2, sizeof title - 1);
    ok = ok && std::fwrite(title, 80, 1, f) == 1;
    put_i32(f, 164, ok);
    put_i32(f, 4, ok);
    put_i32(f, N, ok);
    put_i32(f, 4, ok);
    return std::fclose(f) == 0 && ok;
}

// one DCD frame of n beads from Coord AoS c (components a, b, d of 7)
bool append_frame(const std::string &path, const float *c, int n, int a, int b, int d, std::vector<float> &tmp) {
    FILE *f = std::fopen(path.c_str(), "a");
    if (!f) return false;
    tmp.resize(n);
    bool ok = true;
    for (int comp : {a, b, d}) {
        for (int i = 0; i < n; i++) tmp[i] = c[7 * (size_t)i + comp];
        put_i32(f, 4 * n, ok);
        ok = ok && (n == 0 || std::fwrite(tmp.data(), 4, n, f) == (size_t)n);
        put_i32(f, 4 * n, ok);
    }
    return std::fclose(f) == 0 && ok;
}

void writer_loop(mtg_output *o) {
    cudaSetDevice(o->device);
    std::vector<float> tmp;
    for (;;) {
        mtg_output::Job job;
        {
            std::unique_lock<std::mutex> lk(o->m);
            o->cv.wait(lk, [o] { return o->stop || !o->jobs.empty(); });
            if (o->jobs.empty()) return;
            job = o->jobs.front();
            o->jobs.pop_front();
        }
        bool ok = cudaEventSynchronize(o->copied[job.slot]) == cudaSuccess;
        const char *why = ok ? nullptr : "copy of a stride frame failed";
        if (ok && job.frame) {
            for (int t = 0; t < o->nt && ok; t++) {
                const float *c = o->h_coords[job.slot] + 7 * (size_t)o->off[t];
                const int n = o->off[t + 1] - o->off[t];
                // xyz file: (x, y, z); angle file: (fi, psi, theta) (src/preparator.cpp:583-601)
                ok = append_frame(o->xyz[t], c, n, 0, 1, 2, tmp) && append_frame(o->ang[t], c, n, 3, 5, 4, tmp);
            }
            if (!ok) why = "writing a DCD frame failed";
        }
        if (ok && job.energies) {
            const double *E = o->h_en[job.slot];
            for (int t = 0; t < o->nt; t++) {
                const double *u = E + 7 * (size_t)t;
                // (src/updater.cpp:28-36): the NaN notice, then the line
                if (!std::isfinite(u[0]) || !std::isfinite(u[1]) || !std::isfinite(u[2]) || !std::isfinite(u[6]))
                    std::fprintf(o->energy_out, "Some energy in %d trajectory is NaN. NOT Exit program\n", t);
                std::fprintf(o->energy_out, "Energies[%d]:\t%f\t%f\t%f\t%f\t%f\t%f\t%f\n", t, u[0], u[1], u[2], u[3],
                             u[4], u[5], u[6]);
            }
            std::fflush(o->energy_out);
        }
        std::lock_guard<std::mutex> lk(o->m);
        if (!ok && !o->error) {
            o->error = MTG_E_CONFIG;
            o->error_msg = why;
        }
        if (job.frame && ok) o->frames_written++;
        o->busy[job.slot] = false;
        o->cv.notify_all();
    }
}

void release(mtg_output *o) {
    if (!o) return;
    if (o->writer.joinable()) {
        {
            std::lock_guard<std::mutex> lk(o->m);
            o->stop = true;
        }
        o->cv.notify_all();
        o->writer.join();
    }
    for (int s = 0; s < mtg_output::kSlots; s++) {
        if (o->d_stage[s]) cudaFree(o->d_stage[s]);
        if (o->d_en[s]) cudaFree(o->d_en[s]);
        if (o->h_coords[s]) cudaFreeHost(o->h_coords[s]);
        if (o->h_en[s]) cudaFreeHost(o->h_en[s]);
        if (o->converted[s]) cudaEventDestroy(o->converted[s]);
        if (o->copied[s]) cudaEventDestroy(o->copied[s]);
    }
    if (o->d_ignored_err) cudaFree(o->d_ignored_err);
    if (o->energy_out && o->energy_out != stdout) std::fclose(o->energy_out);
    if (o->copy) cudaStreamDestroy(o->copy);
    delete o;
}

#define OCK(call)                                                                          \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            release(o);                                                                    \
            return mtg_internal_fail(MTG_E_CUDA, cudaGetErrorString(e_));                 \
        }                                                                                  \
    } while (0)

}  // namespace

void mtg_internal_close_output(mtg_engine *e) {
    if (e && e->output) {
        release(e->output);
        e->output = nullptr;
    }
}

extern "C" {

int mtg_output_open(mtg_engine *e, const char *const *xyz_paths, const char *const *ang_paths, int nfile, int npriv,
                    int nsavc, float delta, const char *remark2, const char *energy_path) {
    if (!e || !xyz_paths || !ang_paths) return mtg_internal_fail(MTG_E_CONFIG, "engine or paths is NULL");
    if (e->output) return mtg_internal_fail(MTG_E_STATE, "output already open");
    cudaSetDevice(e->device);
    char date[80];
    if (!remark2) {
        const std::time_t now = std::time(nullptr);
        std::snprintf(date, sizeof date, "REMARKS DATE: %s", std::asctime(std::localtime(&now)));
        remark2 = date;
    }
    auto *o = new mtg_output();
    o->device = e->device;
    o->nb = e->nb;
    o->nt = e->nt;
    o->off = e->h_off;
    for (int t = 0; t < e->nt; t++) {
        if (!xyz_paths[t] || !ang_paths[t]) {
            release(o);
            return mtg_internal_fail(MTG_E_CONFIG, "a DCD path is NULL");
        }
        o->xyz.emplace_back(xyz_paths[t]);
        o->ang.emplace_back(ang_paths[t]);
        const int n = e->h_off[t + 1] - e->h_off[t];
        if (!write_header(xyz_paths[t], n, nfile, npriv, nsavc, delta, remark2) ||
            !write_header(ang_paths[t], n, nfile, npriv, nsavc, delta, remark2)) {
            release(o);
            return mtg_internal_fail(MTG_E_CONFIG, "cannot write a DCD header");
        }
    }
    OCK(cudaStreamCreateWithFlags(&o->copy, cudaStreamNonBlocking));
    OCK(cudaMalloc(&o->d_ignored_err, sizeof(int)));
    for (int s = 0; s < mtg_output::kSlots; s++) {
        OCK(cudaMalloc(&o->d_stage[s], sizeof(float) * 7 * (size_t)e->nb));
        OCK(cudaMalloc(&o->d_en[s], sizeof(double) * 7 * (size_t)e->nt));
        OCK(cudaMallocHost(&o->h_coords[s], sizeof(float) * 7 * (size_t)e->nb));
        OCK(cudaMallocHost(&o->h_en[s], sizeof(double) * 7 * (size_t)e->nt));
        OCK(cudaEventCreateWithFlags(&o->converted[s], cudaEventDisableTiming));
        OCK(cudaEventCreateWithFlags(&o->copied[s], cudaEventDisableTiming));
    }
    if (energy_path) {
        o->energy_out = std::fopen(energy_path, "a");
        if (!o->energy_out) {
            o->energy_out = stdout;
            release(o);
            return mtg_internal_fail(MTG_E_CONFIG, "cannot open the energy file");
        }
    }
    o->writer = std::thread(writer_loop, o);
    e->output = o;
    return MTG_OK;
}

int mtg_output_frame(mtg_engine *e, long long step, int frame, int energies) {
    if (!e || !e->output) return mtg_internal_fail(MTG_E_STATE, "no output open");
    if (!e->have_state) return mtg_internal_fail(MTG_E_STATE, "no state uploaded");
    mtg_output *o = e->output;
    cudaSetDevice(e->device);
    int slot = -1;
    {
        std::unique_lock<std::mutex> lk(o->m);
        o->cv.wait(lk, [o] { return !o->busy[0] || !o->busy[1] || o->error; });
        if (o->error) return mtg_internal_fail(o->error, o->error_msg.c_str());
        slot = o->busy[0] ? 1 : 0;
        o->busy[slot] = true;
    }
    cudaError_t ce = cudaSuccess;
    if (frame) launch_coords_from_frames(e->kp, e->frame[e->cur], o->d_stage[slot], e->stream);
    if (energies) {
        launch_energy(e->kp, e->bufs(), nullptr, e->en_partials, e->work, e->nwork, e->stream);
        launch_energy_totals(e->kp, e->en_partials, e->work_first, o->d_en[slot], o->d_ignored_err, e->stream);
    }
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaEventRecord(o->converted[slot], e->stream);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(o->copy, o->converted[slot], 0);
    if (ce == cudaSuccess && frame)
        ce = cudaMemcpyAsync(o->h_coords[slot], o->d_stage[slot], sizeof(float) * 7 * (size_t)e->nb,
                             cudaMemcpyDeviceToHost, o->copy);
    if (ce == cudaSuccess && energies)
        ce = cudaMemcpyAsync(o->h_en[slot], o->d_en[slot], sizeof(double) * 7 * (size_t)e->nt,
                             cudaMemcpyDeviceToHost, o->copy);
    if (ce == cudaSuccess) ce = cudaEventRecord(o->copied[slot], o->copy);
    std::lock_guard<std::mutex> lk(o->m);
    if (ce != cudaSuccess) {
        o->busy[slot] = false;
        return mtg_internal_fail(MTG_E_CUDA, cudaGetErrorString(ce));
    }
    o->jobs.push_back({slot, step, frame != 0, energies != 0});
    o->cv.notify_all();
    return MTG_OK;
}

int mtg_output_flush(mtg_engine *e, long long *frames_written) {
    if (!e || !e->output) return mtg_internal_fail(MTG_E_STATE, "no output open");
    mtg_output *o = e->output;
    std::unique_lock<std::mutex> lk(o->m);
    o->cv.wait(lk, [o] { return (o->jobs.empty() && !o->busy[0] && !o->busy[1]) || o->error; });
    if (frames_written) *frames_written = o->frames_written;
    if (o->error) return mtg_internal_fail(o->error, o->error_msg.c_str());
    return MTG_OK;
}

int mtg_output_close(mtg_engine *e) {
    if (!e || !e->output) return MTG_OK;
    int rc = MTG_OK;
    {
        mtg_output *o = e->output;
        std::unique_lock<std::mutex> lk(o->m);
        o->cv.wait(lk, [o] { return (o->jobs.empty() && !o->busy[0] && !o->busy[1]) || o->error; });
        if (o->error) rc = mtg_internal_fail(o->error, o->error_msg.c_str());
    }
    mtg_internal_close_output(e);
    return rc;
}

}  // extern "C"
