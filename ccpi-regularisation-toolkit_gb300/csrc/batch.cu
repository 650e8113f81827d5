// Batched regularisation of many volumes of uneven shape (FGP-TV and TGV).
//
// All volumes advance together, driven by a device-resident descriptor table
// (dims, state pointers, lambda, stop control) and a tile -> volume map, and
// every volume keeps its own stopping rule.  Three schedules:
//   * graph: each iteration is ONE kernel launch (two for 2D TGV) over a flat
//     grid of every volume's tiles, a finalize CTA per volume on check
//     iterations; the whole loop is captured into one CUDA graph and launched
//     once (CILREG_BATCH_GRAPH=0: plain launches);
//   * graph of two-voxel launches (FGP, volumes with even x extents and
//     8-byte aligned arrays): the same with the tiles of k_fgp_x2_batch
//     (fgp_x2.cu), two voxels per thread; chosen when every volume's single
//     call runs the two-voxel kernel, so that a batch equals its single calls
//     bit for bit;
//   * persistent (FGP): one launch runs every iteration of every volume; its
//     CTAs take (iteration, tile) items from a device-side queue and wait
//     only for their own volume's previous iteration (k_fgp_persistent,
//     fgp_tiled.cu), optionally in groups of volumes whose state fits in L2.
// An autotuner (on by default for 3D FGP batches of 8 or more iterations;
// CILREG_BATCH_AUTOTUNE=0 turns it off) times three iterations of each
// candidate schedule and z chunk on the batch itself and keeps the fastest,
// per GPU name and batch shape, in the process and in a cache file
// (CILREG_AUTOTUNE_CACHE, default ~/.cache/cilreg-gb300/autotune.tsv; an
// empty value keeps it in the process only).  CILREG_BATCH_MODE=graph, x2 or
// persistent fixes the schedule ("persistent:<MB>" with volume groups of at
// most that many MB of state).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <sys/stat.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cilreg_gb300.h"
#include "drivers.cuh"
#include "fgp_tiled.cuh"
#include "tgv_batch.cuh"
#include "tgv_tiled.cuh"
#include "nvtx.cuh"

namespace cilreg {
namespace {

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct BatchLayout {
    std::vector<Dims> dims;
    bool three = false;
};

int read_dims(int nvol, const int* dims, BatchLayout& L) {
    if (nvol < 1) return fail(ERR_ARG, __FILE__, __LINE__, "empty batch");
    if (!dims) return fail(ERR_ARG, __FILE__, __LINE__, "null dims");
    L.dims.resize(nvol);
    int n3 = 0;
    for (int v = 0; v < nvol; v++) {
        CILREG_TRY(check_dims(dims[3 * v], dims[3 * v + 1], dims[3 * v + 2]));
        L.dims[v] = make_dims(dims[3 * v], dims[3 * v + 1], dims[3 * v + 2] < 1 ? 1 : dims[3 * v + 2]);
        n3 += L.dims[v].nz > 1;
    }
    if (n3 != 0 && n3 != nvol)
        return fail(ERR_ARG, __FILE__, __LINE__, "a batch must be all 2D or all 3D (%d of %d are 3D)", n3, nvol);
    L.three = n3 == nvol;
    return OK;
}

bool env_flag(const char* name, bool dflt) {
    const char* e = getenv(name);
    if (!e || !*e) return dflt;
    return e[0] != '0';
}

// --------------------------------------------------------------------------
// z-chunk autotuning cache
std::mutex g_tune_lock;
std::map<std::string, int> g_tune;

std::string tune_key(const char* alg, const BatchLayout& L) {
    cudaDeviceProp prop;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaGetDeviceProperties(&prop, dev);
    std::string k = std::string(alg) + "|" + prop.name + "|";
    for (const Dims& d : L.dims) {
        char b[64];
        snprintf(b, sizeof(b), "%dx%dx%d;", d.nx, d.ny, d.nz);
        k += b;
    }
    return k;
}

// the autotuner's cache file ("" when the cache stays in the process)
std::string tune_cache_path() {
    const char* e = getenv("CILREG_AUTOTUNE_CACHE");
    if (e) return std::string(e);
    std::string dir;
    if (const char* x = getenv("XDG_CACHE_HOME")) dir = x;
    else if (const char* h = getenv("HOME")) dir = std::string(h) + "/.cache";
    else return "";
    mkdir(dir.c_str(), 0755);
    dir += "/cilreg-gb300";
    mkdir(dir.c_str(), 0755);
    return dir + "/autotune.tsv";
}

int cached_choice(const std::string& key) {
    std::lock_guard<std::mutex> g(g_tune_lock);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return it->second;
    const std::string cpath = tune_cache_path();
    const char* path = cpath.empty() ? nullptr : cpath.c_str();
    if (path) {
        FILE* fp = fopen(path, "r");
        if (fp) {
            char line[8192];
            while (fgets(line, sizeof(line), fp)) {
                char* tab = strrchr(line, '\t');
                if (!tab) continue;
                *tab = 0;
                if (key == line) {
                    int z = atoi(tab + 1);
                    fclose(fp);
                    g_tune[key] = z;
                    return z;
                }
            }
            fclose(fp);
        }
    }
    return 0;
}

void store_choice(const std::string& key, int z) {
    std::lock_guard<std::mutex> g(g_tune_lock);
    g_tune[key] = z;
    const std::string cpath = tune_cache_path();
    const char* path = cpath.empty() ? nullptr : cpath.c_str();
    if (path) {
        FILE* fp = fopen(path, "a");
        if (fp) {
            fprintf(fp, "%s\t%d\n", key.c_str(), z);
            fclose(fp);
        }
    }
}

// --------------------------------------------------------------------------
// FGP batch
struct FgpBatch {
    std::vector<FgpBatchVol> vols;
    std::vector<int> tile_vol;
    std::vector<CheckSlot> slots;
    FgpBatchVol* d_vols = nullptr;
    int* d_tile_vol = nullptr;
    CheckSlot* d_slots = nullptr;
    StopCtl** d_ctlp = nullptr;
    StopCtl* d_ctl = nullptr;
    float* ring = nullptr;
    size_t ring_bytes = 0;
    long long ntiles = 0;
    bool wide = false;  // some volume has 2^31 voxels or more
    bool x2 = false;    // two-voxel tiles (k_fgp_x2_batch)
};

int fgp_build(FgpBatch& B, Scratch& sc, const BatchLayout& L, const float* const* f, float* const* u,
              const float* lams, int zc_override, cudaStream_t s, bool x2 = false) {
    const int nvol = (int)L.dims.size();
    const int nc = L.three ? 3 : 2;
    B.x2 = x2;
    B.vols.assign(nvol, FgpBatchVol());
    B.ntiles = 0;
    size_t ring_floats = 0;
    for (int v = 0; v < nvol; v++) {
        const Dims& d = L.dims[v];
        FgpBatchVol& V = B.vols[v];
        V.d = d;
        if (d.n >= (1LL << 31)) B.wide = true;
        V.zc = zc_override > 0 ? (d.nz > 1 ? (zc_override < d.nz ? zc_override : d.nz) : 1) : fgp_default_zchunk(d);
        if (x2)
            fgp_x2_tile_grid(d, V.zc, V.gx, V.gy, V.gz);
        else
            fgp_tile_grid(d, V.zc, V.gx, V.gy, V.gz);
        V.tile_base = B.ntiles;
        B.ntiles += (long long)V.gx * V.gy * V.gz;
        ring_floats += align256(sizeof(float) * (size_t)d.n) / sizeof(float) * 3 * nc;
    }
    if (B.ntiles > 2147483647LL) return fail(ERR_ARG, __FILE__, __LINE__, "batch too large (%lld tiles)", B.ntiles);
    B.ring_bytes = ring_floats * sizeof(float);
    B.ring = (float*)sc.bytes(B.ring_bytes);
    double2* part = (double2*)sc.bytes(sizeof(double2) * (size_t)B.ntiles);
    B.d_ctl = (StopCtl*)sc.bytes(sizeof(StopCtl) * nvol);
    B.d_vols = (FgpBatchVol*)sc.bytes(sizeof(FgpBatchVol) * nvol);
    B.d_tile_vol = (int*)sc.bytes(sizeof(int) * (size_t)B.ntiles);
    B.d_slots = (CheckSlot*)sc.bytes(sizeof(CheckSlot) * nvol);
    B.d_ctlp = (StopCtl**)sc.bytes(sizeof(StopCtl*) * nvol);
    if (!B.ring || !part || !B.d_ctl || !B.d_vols || !B.d_tile_vol || !B.d_slots || !B.d_ctlp) return sc.status();
    B.tile_vol.resize(B.ntiles);
    B.slots.resize(nvol);
    std::vector<StopCtl*> ctlp(nvol);
    float* r = B.ring;
    for (int v = 0; v < nvol; v++) {
        FgpBatchVol& V = B.vols[v];
        const size_t stride = align256(sizeof(float) * (size_t)V.d.n) / sizeof(float);
        for (int b = 0; b < 3; b++)
            for (int c = 0; c < 3; c++) {
                if (c < nc) {
                    V.ring[b][c] = r;
                    r += stride;
                } else {
                    V.ring[b][c] = nullptr;
                }
            }
        V.f = f[v];
        V.u = u[v];
        V.lam = lams[v];
        V.multip = L.three ? (1.0f / (12.0f * V.lam)) : (1.0f / (8.0f * V.lam));
        V.ctl = B.d_ctl + v;
        V.partials = part + V.tile_base;
        const long long nt = (long long)V.gx * V.gy * V.gz;
        for (long long t = 0; t < nt; t++) B.tile_vol[V.tile_base + t] = v;
        B.slots[v] = CheckSlot{V.partials, nt, V.ctl};
        ctlp[v] = V.ctl;
    }
    CILREG_CUDA(cudaMemcpyAsync(B.d_vols, B.vols.data(), sizeof(FgpBatchVol) * nvol, cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(B.d_tile_vol, B.tile_vol.data(), sizeof(int) * (size_t)B.ntiles,
                                cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(B.d_slots, B.slots.data(), sizeof(CheckSlot) * nvol, cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(B.d_ctlp, ctlp.data(), sizeof(StopCtl*) * nvol, cudaMemcpyHostToDevice, s));
    // the host vectors must outlive the copies
    CILREG_CUDA(cudaStreamSynchronize(s));
    return OK;
}

int fgp_reset(FgpBatch& B, int nvol, int iters, cudaStream_t s) {
    CILREG_CUDA(cudaMemsetAsync(B.ring, 0, B.ring_bytes, s));
    return launch_init_ctls(B.d_ctlp, nvol, iters, s);
}

int fgp_enqueue(FgpBatch& B, int nvol, bool three, int iters, float epsil, int methodTV, int nonneg, cudaStream_t s) {
    float tk = 1.0f, cprev = 0.0f;
    const bool checking = epsil != 0.0f;
    for (int it = 0; it < iters; it++) {
        const int check = (checking && it % 5 == 0) ? 1 : 0;
        const int write_u = (it == iters - 1) || check || (checking && (it + 1) % 5 == 0);
        const int write_p = (it != iters - 1);
        if (B.x2)
            CILREG_TRY(fgp_x2_batch_step(B.d_vols, B.d_tile_vol, B.ntiles, it, cprev, nonneg == 1, methodTV != 0,
                                         write_u, write_p, check, s));
        else
            CILREG_TRY(fgp_batch_step(B.d_vols, B.d_tile_vol, B.ntiles, three, B.wide, it, cprev, nonneg == 1,
                                      methodTV != 0, write_u, write_p, check, s));
        note_launch();
        const float tkp1 = (1.0f + sqrtf(1.0f + 4.0f * tk * tk)) * 0.5f;  // FGP_TV_core.c:138
        cprev = (tk - 1.0f) / tkp1;
        tk = tkp1;
        if (check) CILREG_TRY(launch_finalize_batch(B.d_slots, nvol, epsil, it, s));
    }
    return OK;
}

// run the enqueued loop through one CUDA graph (capture, instantiate, launch)
template <class Enq>
int run_graph(cudaStream_t s, Enq enqueue) {
    CILREG_RANGE("cilreg graph launch");
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    CILREG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue();
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (rc != 0) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    CILREG_CUDA(e);
    e = cudaGraphInstantiate(&ge, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        CILREG_CUDA(e);
    }
    e = cudaGraphLaunch(ge, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaGraphExecDestroy(ge);
    cudaGraphDestroy(g);
    CILREG_CUDA(e);
    CILREG_CUDA(e2);
    return OK;
}

int read_infos(const StopCtl* d_ctl, int nvol, float* infos, cudaStream_t s) {
    std::vector<StopCtl> h(nvol);
    CILREG_CUDA(cudaMemcpyAsync(h.data(), d_ctl, sizeof(StopCtl) * nvol, cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    if (infos)
        for (int v = 0; v < nvol; v++) {
            infos[2 * v] = (float)h[v].iters;
            infos[2 * v + 1] = h[v].re;
        }
    return OK;
}

// One persistent launch for every iteration of every volume.  group_mb > 0
// cuts the volumes (in order) into groups of at most that much FGP state
// (44 B per voxel), run one group after another so that a small group's
// state stays in L2 across its iterations; 0 runs all volumes as one group.
// Items of iterations it0 .. it0 + nits - 1 of a run of `iters`; with
// ran_out, a wait that gives up is reported there instead of failing.
int fgp_persistent_enqueue(FgpBatch& B, const BatchLayout& L, int it0, int nits, int iters, float epsil,
                           int methodTV, int nonneg, int group_mb, long long wait_limit, cudaStream_t s, Scratch& sc,
                           int* ran_out = nullptr) {
    const int nvol = (int)L.dims.size();
    std::vector<long long> gtile{0}, gitem{0};
    double acc = 0.0;
    for (int v = 0; v < nvol; v++) {
        const double bytes = 44.0 * (double)L.dims[v].n;
        if (group_mb > 0 && acc > 0.0 && acc + bytes > (double)group_mb * 1048576.0) {
            gtile.push_back(B.vols[v].tile_base);
            gitem.push_back(gitem.back() + (long long)nits * (gtile.back() - gtile[gtile.size() - 2]));
            acc = 0.0;
        }
        acc += bytes;
    }
    gtile.push_back(B.ntiles);
    gitem.push_back(gitem.back() + (long long)nits * (gtile.back() - gtile[gtile.size() - 2]));
    const int ngroups = (int)gtile.size() - 1;
    std::vector<float> carr(iters > 0 ? iters : 1);
    float tk = 1.0f, cprev = 0.0f;
    for (int it = 0; it < iters; it++) {
        carr[it] = cprev;
        const float tkp1 = (1.0f + sqrtf(1.0f + 4.0f * tk * tk)) * 0.5f;  // FGP_TV_core.c:138
        cprev = (tk - 1.0f) / tkp1;
        tk = tkp1;
    }
    // queue counter, error flag, per-volume arrivals and releases: zeroed together
    const size_t ctl_bytes = align256(sizeof(unsigned long long) * (1 + (size_t)nvol) + sizeof(int) * (1 + (size_t)nvol));
    unsigned char* ctl = (unsigned char*)sc.bytes(ctl_bytes);
    float* d_carr = sc.floats(iters > 0 ? iters : 1);
    long long* d_g = (long long*)sc.bytes(sizeof(long long) * 2 * (size_t)(ngroups + 1));
    if (!ctl || !d_carr || !d_g) return sc.status();
    CILREG_CUDA(cudaMemsetAsync(ctl, 0, ctl_bytes, s));
    std::vector<long long> g(gtile);
    g.insert(g.end(), gitem.begin(), gitem.end());
    CILREG_CUDA(cudaMemcpyAsync(d_carr, carr.data(), sizeof(float) * carr.size(), cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(d_g, g.data(), sizeof(long long) * g.size(), cudaMemcpyHostToDevice, s));
    FgpPersistArgs A;
    A.vols = B.d_vols;
    A.tile_vol = B.d_tile_vol;
    A.carr = d_carr;
    A.next = (unsigned long long*)ctl;
    A.arrive = A.next + 1;
    A.error = (int*)(A.arrive + nvol);
    A.release = A.error + 1;
    A.gtile = d_g;
    A.gitem = d_g + (ngroups + 1);
    A.ngroups = ngroups;
    A.it0 = it0;
    A.iters = iters;
    A.nonneg = nonneg == 1;
    A.aniso = methodTV != 0;
    A.checking = epsil != 0.0f;
    A.epsil = epsil;
    A.wait_limit = wait_limit;
    const long long items = gitem.back();
    int nctas = fgp_persistent_ctas();
    if ((long long)nctas > items) nctas = (int)items;
    if (items > 0) {
        CILREG_TRY(fgp_persistent_launch(A, L.three, B.wide, nctas, s));
        note_launch();
    }
    int h_err = 0;
    CILREG_CUDA(cudaMemcpyAsync(&h_err, A.error, sizeof(int), cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    // the host buffers must outlive their copies, done by the synchronisation above
    if (ran_out) {
        *ran_out = h_err;
        return OK;
    }
    if (h_err) return fail(ERR_CUDA, __FILE__, __LINE__, "persistent batch: a dependency wait ran out");
    return OK;
}

// schedule of a batched FGP run; code = mode * 100000 + group_mb * 100 + zc
struct FgpSchedule {
    int mode = 0;      // 0 graph of flat-grid launches, 1 persistent kernel, 2 graph of two-voxel launches
    int zc = 0;        // z chunk of the streaming tiles (0: fgp_default_zchunk)
    int group_mb = 0;  // persistent: L2 groups of at most this many MB of state (0: one group)
    int code() const { return mode * 100000 + group_mb * 100 + zc; }
    static FgpSchedule from(int c) {
        FgpSchedule t;
        t.mode = c / 100000;
        t.group_mb = (c / 100) % 1000;
        t.zc = c % 100;
        return t;
    }
};

constexpr long long kWaitLimit = 1LL << 23;  // polls of about 0.2 us: well over a second

int fgp_run_schedule(const FgpSchedule& S, const BatchLayout& L, const float* const* f, float* const* u,
                     const float* lams, int iters, float epsil, int methodTV, int nonneg, float* infos,
                     cudaStream_t s) {
    const int nvol = (int)L.dims.size();
    Scratch sc(s);
    FgpBatch B;
    const bool x2 = S.mode == 2;
    if (x2 && !fgp_x2_batch_usable(L.dims.data(), f, u, nvol))
        return fail(ERR_ARG, __FILE__, __LINE__, "two-voxel batch: a volume has an odd x extent or misaligned arrays");
    CILREG_TRY(fgp_build(B, sc, L, f, u, lams, S.zc, s, x2));
    CILREG_TRY(fgp_reset(B, nvol, iters, s));
    if (S.mode == 1 && iters > 0)
        CILREG_TRY(fgp_persistent_enqueue(B, L, 0, iters, iters, epsil, methodTV, nonneg, S.group_mb, kWaitLimit, s,
                                          sc));
    else if (env_flag("CILREG_BATCH_GRAPH", true) && iters > 0)
        CILREG_TRY(run_graph(s, [&]() { return fgp_enqueue(B, nvol, L.three, iters, epsil, methodTV, nonneg, s); }));
    else
        CILREG_TRY(fgp_enqueue(B, nvol, L.three, iters, epsil, methodTV, nonneg, s));
    return read_infos(B.d_ctl, nvol, infos, s);
}

// pick the schedule: fixed by CILREG_BATCH_MODE, else the cached or freshly
// timed fastest candidate for 3D batches, else one graph of launches
int fgp_choose_schedule(const BatchLayout& L, const float* const* f, float* const* u, const float* lams, int iters,
                        int methodTV, int nonneg, cudaStream_t s, FgpSchedule& out) {
    out = FgpSchedule();
    const int nvol = (int)L.dims.size();
    // A batch gives its volumes' single-call results bit for bit: when every
    // volume's single call runs the two-voxel kernel (fgp.cu: 3D, even rows,
    // 2^21 voxels up to the tensor-copy kernel's sizes), the batch runs
    // two-voxel tiles; otherwise the one-voxel schedules, whose arithmetic is
    // that of the streaming and tensor-copy kernels.
    bool all_x2 = fgp_x2_batch_usable(L.dims.data(), f, u, nvol);
    for (int v = 0; v < nvol && all_x2; v++) all_x2 = !fgp_tma_usable(L.dims[v]) && fgp_x2_plan(L.dims[v]).use;
    if (const char* m = getenv("CILREG_BATCH_MODE")) {
        // "graph", "x2" (graph of two-voxel launches), "persistent" or
        // "persistent:<MB>" (volume groups of at most MB of state)
        if (m[0] == 'p') {
            out.mode = 1;
            if (const char* c = strchr(m, ':')) out.group_mb = atoi(c + 1) < 0 ? 0 : atoi(c + 1) % 1000;
        } else if (m[0] == 'x' && fgp_x2_batch_usable(L.dims.data(), f, u, nvol)) {
            out.mode = 2;
        }
        return OK;
    }
    if (all_x2) out.mode = 2;
    if (!L.three || iters < 8 || !env_flag("CILREG_BATCH_AUTOTUNE", true)) return OK;
    const std::string key = tune_key("fgp-schedule", L);
    const int c = cached_choice(key);
    if (c != 0) {
        out = FgpSchedule::from(c);
        // the cache key holds the extents only: keep the family of kernels
        // this call's volumes and arrays give
        if (all_x2 && out.mode != 2) {
            out.mode = 2;
            out.group_mb = 0;
        } else if (!all_x2 && out.mode == 2) {
            out.mode = 0;
        }
        return OK;
    }
    std::vector<FgpSchedule> cand;
    for (int mode : {0, 1, 2}) {
        if ((mode == 2) != all_x2) continue;
        for (int zc : {64, 32, 16}) {
            FgpSchedule t;
            t.mode = mode;
            t.zc = zc;
            cand.push_back(t);
        }
    }
    if (!all_x2) {
        FgpSchedule grouped;
        grouped.mode = 1;
        grouped.zc = 16;
        grouped.group_mb = 96;
        cand.push_back(grouped);
    }
    float best = 1e30f;
    cudaEvent_t e0, e1;
    CILREG_CUDA(cudaEventCreate(&e0));
    CILREG_CUDA(cudaEventCreate(&e1));
    int rc = OK;
    for (const FgpSchedule& t : cand) {
        float ms = 0.f;
        for (int rep = 0; rep < 2 && rc == OK; rep++) {  // the first run also warms the pool
            cudaEventRecord(e0, s);
            rc = fgp_run_schedule(t, L, f, u, lams, 3, 0.0f, methodTV, nonneg, nullptr, s);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms, e0, e1);
        }
        if (rc != OK) break;
        if (ms < best) {
            best = ms;
            out = t;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CILREG_TRY(rc);
    store_choice(key, out.code());
    return OK;
}

int fgp_batch_run(int nvol, const float* const* f, float* const* u, const int* dims, const float* lams, int iters,
                  float epsil, int methodTV, int nonneg, float* infos, cudaStream_t caller) {
    CILREG_RANGE("cilreg FGP-TV batch");
    BatchLayout L;
    CILREG_TRY(read_dims(nvol, dims, L));
    if (!f || !u || !lams) return fail(ERR_ARG, __FILE__, __LINE__, "null batch arrays");
    for (int v = 0; v < nvol; v++)
        if (!f[v] || !u[v] || f[v] == u[v]) return fail(ERR_ARG, __FILE__, __LINE__, "bad buffers of volume %d", v);
    int dev = 0;
    CILREG_CUDA(cudaGetDevice(&dev));
    CILREG_TRY(use_device(dev));
    CILREG_CUDA(cudaStreamSynchronize(caller));  // inputs written on the caller's stream are ready
    cudaStream_t s = thread_stream(dev);
    FgpSchedule S;
    CILREG_TRY(fgp_choose_schedule(L, f, u, lams, iters, methodTV, nonneg, s, S));
    return fgp_run_schedule(S, L, f, u, lams, iters, epsil, methodTV, nonneg, infos, s);
}

// --------------------------------------------------------------------------
// TGV batch, 3D: one fused pass per iteration (tgv_fused.cu) over every
// volume's double-buffered state
int tgv_batch_run_fused(int nvol, const float* const* f, float* const* u, const BatchLayout& L, const float* lams,
                        float alpha1, float alpha0, int iters, float L2, float epsil, float* infos, cudaStream_t s) {
    Scratch sc(s);
    const float tau = (float)pow((double)L2, -0.5);  // TGV_core.c:54-55
    std::vector<TgvFusedVol> vols(nvol);
    long long ntiles = 0;
    size_t state_floats = 0;
    for (int v = 0; v < nvol; v++) {
        TgvFusedVol& V = vols[v];
        V.d = L.dims[v];
        tgv_fused_tiles(V.d, V.gx, V.gy, V.gz, V.zc);
        V.tile_base = ntiles;
        ntiles += (long long)V.gx * V.gy * V.gz;
        // two copies of V (3), P (3), Q (6) and a second U
        state_floats += align256(sizeof(float) * (size_t)V.d.n) / sizeof(float) * (2 * 12 + 1);
    }
    if (ntiles > 2147483647LL) return fail(ERR_ARG, __FILE__, __LINE__, "batch too large (%lld tiles)", ntiles);
    float* state = (float*)sc.bytes(sizeof(float) * state_floats);
    double2* part = (double2*)sc.bytes(sizeof(double2) * (size_t)ntiles);
    StopCtl* d_ctl = (StopCtl*)sc.bytes(sizeof(StopCtl) * nvol);
    TgvFusedVol* d_vols = (TgvFusedVol*)sc.bytes(sizeof(TgvFusedVol) * nvol);
    int* d_tile_vol = (int*)sc.bytes(sizeof(int) * (size_t)ntiles);
    CheckSlot* d_slots = (CheckSlot*)sc.bytes(sizeof(CheckSlot) * nvol);
    StopCtl** d_ctlp = (StopCtl**)sc.bytes(sizeof(StopCtl*) * nvol);
    if (!state || !part || !d_ctl || !d_vols || !d_tile_vol || !d_slots || !d_ctlp) return sc.status();
    std::vector<int> tile_vol(ntiles);
    std::vector<CheckSlot> slots(nvol);
    std::vector<StopCtl*> ctlp(nvol);
    std::vector<float*> ualt(nvol);
    // zero V, P, Q of buffer 0 (the buffers of parity 1 are written before they are read)
    float* r = state;
    for (int v = 0; v < nvol; v++) {
        TgvFusedVol& V = vols[v];
        const size_t n = (size_t)V.d.n, stride = align256(sizeof(float) * n) / sizeof(float);
        float* vb[2][3];
        float* pb[2][3];
        float* qb[2][6];
        for (int b = 0; b < 2; b++) {
            for (int c = 0; c < 3; c++) { vb[b][c] = r; r += stride; }
            for (int c = 0; c < 3; c++) { pb[b][c] = r; r += stride; }
            for (int c = 0; c < 6; c++) { qb[b][c] = r; r += stride; }
        }
        ualt[v] = r;
        r += stride;
        for (int c = 0; c < 3; c++) {
            CILREG_CUDA(cudaMemsetAsync(vb[0][c], 0, sizeof(float) * n, s));
            CILREG_CUDA(cudaMemsetAsync(pb[0][c], 0, sizeof(float) * n, s));
        }
        for (int c = 0; c < 6; c++) CILREG_CUDA(cudaMemsetAsync(qb[0][c], 0, sizeof(float) * n, s));
        CILREG_CUDA(cudaMemcpyAsync(u[v], f[v], sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
        float* ub[2] = {u[v], ualt[v]};
        for (int par = 0; par < 2; par++) {
            TgvFusedArgs& A = V.args[par];
            const int cur = par, nxt = par ^ 1;
            A.u = ub[cur];
            A.un = ub[nxt];
            A.u0 = f[v];
            for (int c = 0; c < 3; c++) {
                A.v[c] = vb[cur][c];
                A.vn[c] = vb[nxt][c];
                A.p[c] = pb[cur][c];
                A.pn[c] = pb[nxt][c];
            }
            for (int c = 0; c < 6; c++) {
                A.q[c] = qb[cur][c];
                A.qn[c] = qb[nxt][c];
            }
            A.lambda = lams[v];
            A.alpha1 = alpha1;
            A.alpha0 = alpha0;
            A.tau = tau;
            A.sigma = tau;
            A.inv_lt = 1.0f / (A.lambda + tau);
        }
        V.ctl = d_ctl + v;
        V.partials = part + V.tile_base;
        const long long nt = (long long)V.gx * V.gy * V.gz;
        for (long long t = 0; t < nt; t++) tile_vol[V.tile_base + t] = v;
        slots[v] = CheckSlot{V.partials, nt, V.ctl};
        ctlp[v] = V.ctl;
    }
    // tensor maps of every volume's input arrays, per parity, when every
    // volume qualifies for the staged pass (else the thread-loading pass runs)
    void* d_maps = nullptr;
    std::vector<unsigned char> maps;
    if (tgv_tma_batch_usable(L.dims.data(), nvol)) {
        const size_t mb = tgv_tma_maps_bytes();
        maps.resize(mb * 2 * (size_t)nvol);
        bool ok = true;
        for (int v = 0; v < nvol && ok; v++)
            for (int par = 0; par < 2 && ok; par++)
                ok = tgv_tma_encode(vols[v].args[par], vols[v].d, maps.data() + mb * (2 * (size_t)v + par));
        if (ok) {
            d_maps = sc.bytes(maps.size());
            if (!d_maps) return sc.status();
            CILREG_CUDA(cudaMemcpyAsync(d_maps, maps.data(), maps.size(), cudaMemcpyHostToDevice, s));
        }
    }
    CILREG_CUDA(cudaMemcpyAsync(d_vols, vols.data(), sizeof(TgvFusedVol) * nvol, cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(d_tile_vol, tile_vol.data(), sizeof(int) * (size_t)ntiles, cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(d_slots, slots.data(), sizeof(CheckSlot) * nvol, cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(d_ctlp, ctlp.data(), sizeof(StopCtl*) * nvol, cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    CILREG_TRY(launch_init_ctls(d_ctlp, nvol, iters, s));
    auto enqueue = [&]() -> int {
        for (int it = 0; it < iters; it++) {
            const int check = (epsil != 0.0f && it % 5 == 0) ? 1 : 0;
            if (d_maps)
                CILREG_TRY(tgv_tma_batch_step(d_vols, d_tile_vol, d_maps, ntiles, it & 1, check, s));
            else
                CILREG_TRY(tgv_fused_batch_step(d_vols, d_tile_vol, ntiles, it & 1, check, s));
            note_launch();
            if (check) CILREG_TRY(launch_finalize_batch(d_slots, nvol, epsil, it, s));
        }
        return OK;
    };
    if (env_flag("CILREG_BATCH_GRAPH", true) && iters > 0)
        CILREG_TRY(run_graph(s, enqueue));
    else
        CILREG_TRY(enqueue());
    // the last iterate of each volume is in the buffer its last iteration wrote
    for (int v = 0; v < nvol && iters > 0; v++) {
        float* ub[2] = {u[v], ualt[v]};
        CILREG_TRY(launch_select_pingpong(d_ctl + v, iters, ub, u[v], L.dims[v].n, s));
    }
    if (d_maps) CILREG_TRY(tgv_tma_status(s));
    return read_infos(d_ctl, nvol, infos, s);
}

// --------------------------------------------------------------------------
// TGV batch
int tgv_batch_run(int nvol, const float* const* f, float* const* u, const int* dims, const float* lams, float alpha1,
                  float alpha0, int iters, float L2, float epsil, float* infos, cudaStream_t caller) {
    CILREG_RANGE("cilreg TGV batch");
    BatchLayout L;
    CILREG_TRY(read_dims(nvol, dims, L));
    if (!f || !u || !lams) return fail(ERR_ARG, __FILE__, __LINE__, "null batch arrays");
    for (int v = 0; v < nvol; v++)
        if (!f[v] || !u[v] || f[v] == u[v]) return fail(ERR_ARG, __FILE__, __LINE__, "bad buffers of volume %d", v);
    int dev = 0;
    CILREG_CUDA(cudaGetDevice(&dev));
    CILREG_TRY(use_device(dev));
    CILREG_CUDA(cudaStreamSynchronize(caller));
    cudaStream_t s = thread_stream(dev);
    Scratch sc(s);
    const int np = L.three ? 3 : 2, nq = L.three ? 6 : 3;
    const float tau = (float)pow((double)L2, -0.5);  // TGV_core.c:54-55

    // primal half: the streaming kernel (tgv_tiled.cu) unless
    // CILREG_TGV_KERNEL=simple or a volume has 2^31 voxels or more
    const char* ek = getenv("CILREG_TGV_KERNEL");
    bool stream_primal = !(ek && ek[0] == 's');
    for (int v = 0; v < nvol; v++)
        if (L.dims[v].n >= (1LL << 31)) stream_primal = false;
    // 3D batches run the fused pass (CILREG_TGV_FUSED=0: the two passes)
    if (L.three && stream_primal && env_flag("CILREG_TGV_FUSED", true))
        return tgv_batch_run_fused(nvol, f, u, L, lams, alpha1, alpha0, iters, L2, epsil, infos, s);
    std::vector<TgvBatchVol> vols(nvol);
    long long ntiles = 0, nptiles = 0;
    size_t state_floats = 0;
    for (int v = 0; v < nvol; v++) {
        const Launch3 P = plan_launch(L.dims[v]);
        TgvBatchVol& V = vols[v];
        V.d = L.dims[v];
        V.gx = P.grid.x;
        V.gy = P.grid.y;
        V.gz = P.grid.z;
        V.kz = P.kz;
        V.tile_base = ntiles;
        ntiles += (long long)V.gx * V.gy * V.gz;
        if (stream_primal) {
            tgv_primal_tiles(V.d, V.pgx, V.pgy, V.pgz, V.pzc);
        } else {
            V.pgx = V.gx;
            V.pgy = V.gy;
            V.pgz = V.gz;
            V.pzc = V.kz;
        }
        V.ptile_base = nptiles;
        nptiles += (long long)V.pgx * V.pgy * V.pgz;
        state_floats += align256(sizeof(float) * (size_t)V.d.n) / sizeof(float) * (2 * np + nq);
    }
    float* state = (float*)sc.bytes(sizeof(float) * state_floats);
    double2* part = (double2*)sc.bytes(sizeof(double2) * (size_t)nptiles);
    StopCtl* d_ctl = (StopCtl*)sc.bytes(sizeof(StopCtl) * nvol);
    TgvBatchVol* d_vols = (TgvBatchVol*)sc.bytes(sizeof(TgvBatchVol) * nvol);
    int* d_tile_vol = (int*)sc.bytes(sizeof(int) * (size_t)ntiles);
    int* d_ptile_vol = stream_primal ? (int*)sc.bytes(sizeof(int) * (size_t)nptiles) : nullptr;
    CheckSlot* d_slots = (CheckSlot*)sc.bytes(sizeof(CheckSlot) * nvol);
    StopCtl** d_ctlp = (StopCtl**)sc.bytes(sizeof(StopCtl*) * nvol);
    if (!state || !part || !d_ctl || !d_vols || !d_tile_vol || !d_slots || !d_ctlp || (stream_primal && !d_ptile_vol))
        return sc.status();
    CILREG_CUDA(cudaMemsetAsync(state, 0, sizeof(float) * state_floats, s));
    std::vector<int> tile_vol(ntiles), ptile_vol(stream_primal ? nptiles : 0);
    std::vector<CheckSlot> slots(nvol);
    std::vector<StopCtl*> ctlp(nvol);
    float* r = state;
    for (int v = 0; v < nvol; v++) {
        TgvBatchVol& V = vols[v];
        const size_t stride = align256(sizeof(float) * (size_t)V.d.n) / sizeof(float);
        TgvArgs& a = V.args;
        for (int c = 0; c < 3; c++) a.p[c] = a.v[c] = nullptr;
        for (int c = 0; c < 6; c++) a.q[c] = nullptr;
        for (int c = 0; c < np; c++) { a.p[c] = r; r += stride; }
        for (int c = 0; c < np; c++) { a.v[c] = r; r += stride; }
        for (int c = 0; c < nq; c++) { a.q[c] = r; r += stride; }
        a.u = u[v];
        a.u0 = f[v];
        a.lambda = lams[v];
        a.alpha1 = alpha1;
        a.alpha0 = alpha0;
        a.tau = tau;
        a.sigma = tau;
        a.inv_lt = 1.0f / (a.lambda + tau);
        a.check = 0;
        V.ctl = d_ctl + v;
        V.partials = part + V.ptile_base;
        const long long nt = (long long)V.gx * V.gy * V.gz;
        for (long long t = 0; t < nt; t++) tile_vol[V.tile_base + t] = v;
        const long long npt = (long long)V.pgx * V.pgy * V.pgz;
        if (stream_primal)
            for (long long t = 0; t < npt; t++) ptile_vol[V.ptile_base + t] = v;
        slots[v] = CheckSlot{V.partials, npt, V.ctl};
        ctlp[v] = V.ctl;
        CILREG_CUDA(cudaMemcpyAsync(u[v], f[v], sizeof(float) * (size_t)V.d.n, cudaMemcpyDeviceToDevice, s));
    }
    CILREG_CUDA(cudaMemcpyAsync(d_vols, vols.data(), sizeof(TgvBatchVol) * nvol, cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(d_tile_vol, tile_vol.data(), sizeof(int) * (size_t)ntiles, cudaMemcpyHostToDevice, s));
    if (stream_primal)
        CILREG_CUDA(cudaMemcpyAsync(d_ptile_vol, ptile_vol.data(), sizeof(int) * (size_t)nptiles,
                                    cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(d_slots, slots.data(), sizeof(CheckSlot) * nvol, cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(d_ctlp, ctlp.data(), sizeof(StopCtl*) * nvol, cudaMemcpyHostToDevice, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    CILREG_TRY(launch_init_ctls(d_ctlp, nvol, iters, s));
    auto enqueue = [&]() -> int {
        for (int it = 0; it < iters; it++) {
            const int check = (epsil != 0.0f && it % 5 == 0) ? 1 : 0;
            CILREG_TRY(tgv_batch_step(d_vols, d_tile_vol, ntiles, d_ptile_vol, nptiles, L.three, check, s));
            note_launch(2);
            if (check) CILREG_TRY(launch_finalize_batch(d_slots, nvol, epsil, it, s));
        }
        return OK;
    };
    if (env_flag("CILREG_BATCH_GRAPH", true) && iters > 0)
        CILREG_TRY(run_graph(s, enqueue));
    else
        CILREG_TRY(enqueue());
    return read_infos(d_ctl, nvol, infos, s);
}

}  // namespace
}  // namespace cilreg

using namespace cilreg;

extern "C" {

int cilreg_fgp_tv_batch_dev(int nvol, const float* const* d_in, float* const* d_out, const int* dims,
                            const float* lambdas, int iters, float epsil, int methodTV, int nonneg, float* infovectors,
                            void* stream) {
    return fgp_batch_run(nvol, d_in, d_out, dims, lambdas, iters, epsil, methodTV, nonneg, infovectors,
                         (cudaStream_t)stream);
}

int cilreg_selftest_batch_wait(int gpu_device, int* ran_out) {
    if (!ran_out) return fail(ERR_ARG, __FILE__, __LINE__, "null result pointer");
    *ran_out = 0;
    CILREG_TRY(use_device(gpu_device));
    cudaStream_t s = thread_stream(gpu_device);
    Scratch sc(s);
    const int dims[3] = {40, 20, 12};
    BatchLayout L;
    CILREG_TRY(read_dims(1, dims, L));
    const long long n = L.dims[0].n;
    float* f = sc.floats(2 * n);
    if (!f) return sc.status();
    float* u = f + n;
    CILREG_CUDA(cudaMemsetAsync(f, 0, sizeof(float) * 2 * n, s));
    const float lam = 0.05f;
    FgpBatch B;
    CILREG_TRY(fgp_build(B, sc, L, &f, &u, &lam, 0, s));
    CILREG_TRY(fgp_reset(B, 1, 2, s));
    // every item of this launch belongs to iteration 1, whose predecessor is
    // never released: each wait polls 4096 times (about a millisecond), gives
    // up, flags the error and its CTA leaves
    int out = 0;
    CILREG_TRY(fgp_persistent_enqueue(B, L, 1, 1, 2, 0.0f, 0, 0, 0, 4096, s, sc, &out));
    // the device still runs work
    CILREG_TRY(fgp_reset(B, 1, 2, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    *ran_out = out;
    return OK;
}

int cilreg_tgv_batch_dev(int nvol, const float* const* d_in, float* const* d_out, const int* dims,
                         const float* lambdas, float alpha1, float alpha0, int iters, float L2, float epsil,
                         float* infovectors, void* stream) {
    return tgv_batch_run(nvol, d_in, d_out, dims, lambdas, alpha1, alpha0, iters, L2, epsil, infovectors,
                         (cudaStream_t)stream);
}

}  // extern "C"
