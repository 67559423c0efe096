// mg_io.cu - the reference's trajectory file (trajectory(), src/dumpxyz.c:37-66) written
// from device-resident runs, and its checkpoint file (saveit()/loadit(),
// src/loadsave.c:19-128).
//
// Trajectory frames leave the device without stalling the integrator: at a frame the
// compute stream copies the positions into one of two device staging buffers (a
// device-to-device copy of 24 bytes per site), a copy stream moves that buffer into the
// matching pinned host buffer, and a writer thread waits for the copy and appends the
// frame to the file. The integrator only waits when both buffers are still in flight.
// Byte layout (the reference's fwrite calls, native endianness):
//   header, once: int nspecie, nmole, natom; per species int nmole, natom and per
//                 template site char name[5], double aw;
//   per frame:    int nmole_per_specie[nspecie]; double x[natom], y[natom], z[natom].
#include <stdio.h>
#include <string.h>

#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "mg_internal.cuh"

struct MgTraj {
    FILE *fp = nullptr;
    int every = 0;
    long long istep = 0;
    long long enqueued = 0, written = 0;
    int natom = 0;
    std::vector<int> nmole;
    cudaStream_t copy = nullptr;
    double *d_stage[2] = {nullptr, nullptr};
    double *h_pin[2] = {nullptr, nullptr};
    cudaEvent_t staged[2], copied[2];
    bool events = false;
    bool busy[2] = {false, false};
    int next = 0;
    std::thread writer;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<int> queue;
    bool stop = false, failed = false;
    int device = 0;
};

static void traj_writer(MgTraj *t) {
    cudaSetDevice(t->device);
    for (;;) {
        int slot;
        {
            std::unique_lock<std::mutex> lk(t->mu);
            t->cv.wait(lk, [t] { return t->stop || !t->queue.empty(); });
            if (t->queue.empty()) return;  // stop requested and nothing left
            slot = t->queue.front();
            t->queue.pop_front();
        }
        bool ok = cudaEventSynchronize(t->copied[slot]) == cudaSuccess;
        ok = ok && fwrite(t->nmole.data(), sizeof(int), t->nmole.size(), t->fp) == t->nmole.size();
        ok = ok && fwrite(t->h_pin[slot], sizeof(double), 3 * (size_t)t->natom, t->fp) == 3 * (size_t)t->natom;
        {
            std::lock_guard<std::mutex> lk(t->mu);
            t->busy[slot] = false;
            if (ok) t->written++;
            else t->failed = true;
        }
        t->cv.notify_all();
    }
}

static void traj_free(MgTraj *t) {
    if (t->writer.joinable()) {
        {
            std::lock_guard<std::mutex> lk(t->mu);
            t->stop = true;
        }
        t->cv.notify_all();
        t->writer.join();
    }
    for (int i = 0; i < 2; i++) {
        if (t->d_stage[i]) cudaFree(t->d_stage[i]);
        if (t->h_pin[i]) cudaFreeHost(t->h_pin[i]);
    }
    if (t->events)
        for (int i = 0; i < 2; i++) {
            cudaEventDestroy(t->staged[i]);
            cudaEventDestroy(t->copied[i]);
        }
    if (t->copy) cudaStreamDestroy(t->copy);
    if (t->fp) fclose(t->fp);
    delete t;
}

// queues one frame of the device positions d_x ([3][n]) on the context's stream
static mg_status traj_enqueue(mg_ctx *c, const double *d_x) {
    MgTraj *t = c->traj;
    const int slot = t->next;
    t->next ^= 1;
    {
        std::unique_lock<std::mutex> lk(t->mu);
        t->cv.wait(lk, [t, slot] { return !t->busy[slot] || t->failed; });
        if (t->failed) return mg_fail(c, MG_ERR_INVALID, "trajectory: writing a frame failed");
        t->busy[slot] = true;
    }
    const size_t bytes = sizeof(double) * 3 * (size_t)t->natom;
    MG_CUDA(cudaMemcpyAsync(t->d_stage[slot], d_x, bytes, cudaMemcpyDeviceToDevice, c->stream));
    MG_CUDA(cudaEventRecord(t->staged[slot], c->stream));
    MG_CUDA(cudaStreamWaitEvent(t->copy, t->staged[slot], 0));
    MG_CUDA(cudaMemcpyAsync(t->h_pin[slot], t->d_stage[slot], bytes, cudaMemcpyDeviceToHost, t->copy));
    MG_CUDA(cudaEventRecord(t->copied[slot], t->copy));
    {
        std::lock_guard<std::mutex> lk(t->mu);
        t->queue.push_back(slot);
    }
    t->cv.notify_all();
    t->enqueued++;
    return MG_OK;
}

mg_status mg_traj_start(mg_ctx *c, const double *d_x) {
    if (!c->traj || c->traj->enqueued > 0) return MG_OK;
    return traj_enqueue(c, d_x);  // the frame before the first step (src/mspms2.c:57-60)
}

mg_status mg_traj_tick(mg_ctx *c, const double *d_x) {
    MgTraj *t = c->traj;
    if (!t) return MG_OK;
    t->istep++;
    if (t->istep % t->every != 0) return MG_OK;  // src/mspms2.c:123-126
    return traj_enqueue(c, d_x);
}

void mg_traj_destroy(mg_ctx *c) {
    if (c->traj) traj_free(c->traj);
    c->traj = nullptr;
}

extern "C" mg_status mg_traj_open(mg_ctx *c, const char *path, int every, const char *atom_names) {
    if (!c || !path || every < 1 || !atom_names) return MG_ERR_INVALID;
    if (!c->have_topology) return mg_fail(c, MG_ERR_STATE, "set the topology before opening a trajectory");
    mg_traj_destroy(c);
    cudaSetDevice(c->device);
    MgTraj *t = new MgTraj();
    t->device = c->device;
    t->every = every;
    t->natom = c->natom;
    for (int s = 0; s < c->nspecies; s++) t->nmole.push_back(c->species[s].nmole);
    t->fp = fopen(path, "wb");
    if (!t->fp) {
        traj_free(t);
        return mg_fail(c, MG_ERR_INVALID, std::string("trajectory: cannot open ") + path);
    }
    // header (src/dumpxyz.c:42-56)
    const int nmole = c->nmole, natom = c->natom, nsp = c->nspecies;
    bool ok = fwrite(&nsp, sizeof(int), 1, t->fp) == 1 && fwrite(&nmole, sizeof(int), 1, t->fp) == 1 &&
              fwrite(&natom, sizeof(int), 1, t->fp) == 1;
    const char *name = atom_names;
    for (int s = 0; s < nsp && ok; s++) {
        const int nm = c->species[s].nmole, na = c->species[s].natom;
        ok = fwrite(&nm, sizeof(int), 1, t->fp) == 1 && fwrite(&na, sizeof(int), 1, t->fp) == 1;
        for (int a = 0; a < na && ok; a++, name += 5) {
            const double aw = c->h_tmpl_aw[s][a];
            ok = fwrite(name, 1, 5, t->fp) == 5 && fwrite(&aw, sizeof(double), 1, t->fp) == 1;
        }
    }
    const size_t bytes = sizeof(double) * 3 * (size_t)natom;
    bool cuda_ok = ok && cudaStreamCreateWithFlags(&t->copy, cudaStreamNonBlocking) == cudaSuccess;
    for (int i = 0; i < 2 && cuda_ok; i++)
        cuda_ok = cudaMalloc((void **)&t->d_stage[i], bytes) == cudaSuccess &&
                  cudaMallocHost((void **)&t->h_pin[i], bytes) == cudaSuccess;
    if (cuda_ok) {
        cuda_ok = cudaEventCreateWithFlags(&t->staged[0], cudaEventDisableTiming) == cudaSuccess &&
                  cudaEventCreateWithFlags(&t->staged[1], cudaEventDisableTiming) == cudaSuccess &&
                  cudaEventCreateWithFlags(&t->copied[0], cudaEventDisableTiming) == cudaSuccess &&
                  cudaEventCreateWithFlags(&t->copied[1], cudaEventDisableTiming) == cudaSuccess;
        t->events = cuda_ok;
    }
    if (!cuda_ok) {
        traj_free(t);
        return mg_fail(c, ok ? MG_ERR_ALLOC : MG_ERR_INVALID, "trajectory: set-up failed");
    }
    t->writer = std::thread(traj_writer, t);
    c->traj = t;
    return MG_OK;
}

extern "C" mg_status mg_traj_close(mg_ctx *c, long long *nframes) {
    if (!c) return MG_ERR_INVALID;
    if (nframes) *nframes = 0;
    if (!c->traj) return MG_OK;
    MgTraj *t = c->traj;
    {  // drain: the writer takes every queued frame before it stops
        std::lock_guard<std::mutex> lk(t->mu);
        t->stop = true;
    }
    t->cv.notify_all();
    t->writer.join();
    const bool failed = t->failed;
    if (nframes) *nframes = t->written;
    const bool closed = fclose(t->fp) == 0;
    t->fp = nullptr;
    mg_traj_destroy(c);
    if (failed || !closed) return mg_fail(c, MG_ERR_INVALID, "trajectory: writing the file failed");
    return MG_OK;
}

// ---------------------------------------------------------------------------------
// checkpoint: the byte layout of saveit() (src/loadsave.c:19-57)
// ---------------------------------------------------------------------------------
extern "C" mg_status mg_checkpoint_save(const char *path, const mg_checkpoint *k) {
    if (!path || !k || k->natom < 0 || !k->x || !k->y || !k->z || !k->vx || !k->vy || !k->vz) return MG_ERR_INVALID;
    FILE *fp = fopen(path, "wb");
    if (!fp) return MG_ERR_INVALID;
    const size_t n = (size_t)k->natom;
    bool ok = true;
    const double *arr[6] = {k->x, k->y, k->z, k->vx, k->vy, k->vz};
    for (int i = 0; i < 6 && ok; i++) ok = fwrite(arr[i], sizeof(double), n, fp) == n;
    const double sc[15] = {k->qq,  k->ps,  k->gg,  k->ss,    k->qqs,   k->pss,   k->ggs,  k->sss,
                           k->vts, k->rts, k->vbs, k->boxlx, k->boxly, k->boxlz, k->boxv};
    ok = ok && fwrite(sc, sizeof(double), 15, fp) == 15;
    const unsigned char eq = k->equilibrium ? 1 : 0;  // bool, one byte
    ok = ok && fwrite(&eq, 1, 1, fp) == 1;
    ok = ok && fwrite(&k->nframe, sizeof(int), 1, fp) == 1 && fwrite(&k->istep, sizeof(int), 1, fp) == 1;
    ok = ok && fwrite(k->counts, sizeof(int), MG_NCOUNTS, fp) == MG_NCOUNTS;
    ok = ok && fwrite(k->accum, sizeof(double), MG_NCOUNTS, fp) == MG_NCOUNTS;
    ok = (fclose(fp) == 0) && ok;
    return ok ? MG_OK : MG_ERR_INVALID;
}

// loadit() (src/loadsave.c:60-128): the counters only with with_counters (a continued
// run); the kinetic energy, utsbs and the LJ correction are the caller's to recompute
extern "C" mg_status mg_checkpoint_load(const char *path, mg_checkpoint *k, int with_counters) {
    if (!path || !k || k->natom < 0 || !k->x || !k->y || !k->z || !k->vx || !k->vy || !k->vz) return MG_ERR_INVALID;
    FILE *fp = fopen(path, "rb");
    if (!fp) return MG_ERR_INVALID;
    const size_t n = (size_t)k->natom;
    bool ok = true;
    double *arr[6] = {k->x, k->y, k->z, k->vx, k->vy, k->vz};
    for (int i = 0; i < 6 && ok; i++) ok = fread(arr[i], sizeof(double), n, fp) == n;
    double sc[15];
    ok = ok && fread(sc, sizeof(double), 15, fp) == 15;
    if (ok) {
        double *dst[15] = {&k->qq,  &k->ps,  &k->gg,  &k->ss,    &k->qqs,   &k->pss,   &k->ggs,  &k->sss,
                           &k->vts, &k->rts, &k->vbs, &k->boxlx, &k->boxly, &k->boxlz, &k->boxv};
        for (int i = 0; i < 15; i++) *dst[i] = sc[i];
    }
    if (ok && with_counters) {
        unsigned char eq = 0;
        ok = fread(&eq, 1, 1, fp) == 1;
        k->equilibrium = eq ? 1 : 0;
        ok = ok && fread(&k->nframe, sizeof(int), 1, fp) == 1 && fread(&k->istep, sizeof(int), 1, fp) == 1;
        ok = ok && fread(k->counts, sizeof(int), MG_NCOUNTS, fp) == MG_NCOUNTS;
        ok = ok && fread(k->accum, sizeof(double), MG_NCOUNTS, fp) == MG_NCOUNTS;
    }
    fclose(fp);
    return ok ? MG_OK : MG_ERR_INVALID;
}

// the box of a loaded checkpoint: the engine drops everything keyed on the box (cluster
// list, k-vector tables); the Ewald box constants stay as mg_set_params set them, which
// is what the reference's loadit leaves in place
extern "C" mg_status mg_checkpoint_apply(mg_ctx *c, const mg_checkpoint *k) {
    if (!c || !k) return MG_ERR_INVALID;
    if (c->have_topology && k->natom != c->natom) return mg_fail(c, MG_ERR_INVALID, "checkpoint: natom differs");
    mg_status st = mg_set_box(c, k->boxlx, k->boxly, k->boxlz);
    if (st) return st;
    c->list_valid = false;
    c->ewald_box[0] = c->ewald_box[1] = c->ewald_box[2] = 0.0;
    return MG_OK;
}
