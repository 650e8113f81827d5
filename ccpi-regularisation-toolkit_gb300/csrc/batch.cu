// Batched regularisation of many volumes of uneven shape (FGP-TV and TGV).
//
// All volumes advance together: each iteration is ONE kernel launch (two for
// TGV) over a flat grid holding the tiles of every volume, driven by a
// device-resident descriptor table (dims, state pointers, lambda, stop
// control) and a tile -> volume map.  Every volume keeps its own stopping rule
// (one finalize CTA per volume); the tiles of a stopped volume return at once.
// With CILREG_BATCH_GRAPH (default) the whole iteration loop is captured into
// one CUDA graph and launched once.  With CILREG_BATCH_AUTOTUNE the z chunk of
// the FGP streaming kernel is chosen by timing candidate chunks on the batch
// itself; choices are kept per process and optionally in a cache file
// (CILREG_AUTOTUNE_CACHE).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cilreg_gb300.h"
#include "drivers.cuh"
#include "fgp_tiled.cuh"
#include "tgv_batch.cuh"
#include "tgv_tiled.cuh"

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

int cached_choice(const std::string& key) {
    std::lock_guard<std::mutex> g(g_tune_lock);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return it->second;
    const char* path = getenv("CILREG_AUTOTUNE_CACHE");
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
    const char* path = getenv("CILREG_AUTOTUNE_CACHE");
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
};

int fgp_build(FgpBatch& B, Scratch& sc, const BatchLayout& L, const float* const* f, float* const* u,
              const float* lams, int zc_override, cudaStream_t s) {
    const int nvol = (int)L.dims.size();
    const int nc = L.three ? 3 : 2;
    B.vols.assign(nvol, FgpBatchVol());
    B.ntiles = 0;
    size_t ring_floats = 0;
    for (int v = 0; v < nvol; v++) {
        const Dims& d = L.dims[v];
        FgpBatchVol& V = B.vols[v];
        V.d = d;
        if (d.n >= (1LL << 31)) B.wide = true;
        V.zc = zc_override > 0 ? (d.nz > 1 ? (zc_override < d.nz ? zc_override : d.nz) : 1) : fgp_default_zchunk(d);
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
        CILREG_TRY(fgp_batch_step(B.d_vols, B.d_tile_vol, B.ntiles, three, B.wide, it, cprev, nonneg == 1, methodTV != 0,
                                  write_u, write_p, check, s));
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

int fgp_batch_run(int nvol, const float* const* f, float* const* u, const int* dims, const float* lams, int iters,
                  float epsil, int methodTV, int nonneg, float* infos, cudaStream_t caller) {
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
    Scratch sc(s);

    int zc = 0;
    if (L.three && env_flag("CILREG_BATCH_AUTOTUNE", false) && iters >= 8) {
        const std::string key = tune_key("fgp", L);
        zc = cached_choice(key);
        if (zc == 0) {
            // time three iterations for each candidate chunk on the batch itself
            const int cand[3] = {16, 32, 64};
            float best = 1e30f;
            for (int c : cand) {
                Scratch tsc(s);
                FgpBatch T;
                CILREG_TRY(fgp_build(T, tsc, L, f, u, lams, c, s));
                CILREG_TRY(fgp_reset(T, nvol, 3, s));
                cudaEvent_t e0, e1;
                cudaEventCreate(&e0);
                cudaEventCreate(&e1);
                cudaEventRecord(e0, s);
                CILREG_TRY(fgp_enqueue(T, nvol, true, 3, 0.0f, methodTV, nonneg, s));
                cudaEventRecord(e1, s);
                cudaEventSynchronize(e1);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                if (ms < best) {
                    best = ms;
                    zc = c;
                }
            }
            store_choice(key, zc);
        }
    }

    FgpBatch B;
    CILREG_TRY(fgp_build(B, sc, L, f, u, lams, zc, s));
    CILREG_TRY(fgp_reset(B, nvol, iters, s));
    if (env_flag("CILREG_BATCH_GRAPH", true) && iters > 0)
        CILREG_TRY(run_graph(s, [&]() { return fgp_enqueue(B, nvol, L.three, iters, epsil, methodTV, nonneg, s); }));
    else
        CILREG_TRY(fgp_enqueue(B, nvol, L.three, iters, epsil, methodTV, nonneg, s));
    return read_infos(B.d_ctl, nvol, infos, s);
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

int cilreg_tgv_batch_dev(int nvol, const float* const* d_in, float* const* d_out, const int* dims,
                         const float* lambdas, float alpha1, float alpha0, int iters, float L2, float epsil,
                         float* infovectors, void* stream) {
    return tgv_batch_run(nvol, d_in, d_out, dims, lambdas, alpha1, alpha0, iters, L2, epsil, infovectors,
                         (cudaStream_t)stream);
}

}  // extern "C"
