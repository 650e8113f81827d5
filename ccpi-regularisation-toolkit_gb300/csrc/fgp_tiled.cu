// FGP-TV iteration as a 2.5D streaming stencil (2D images are the nz == 1 case).
//
// A CTA of 32 x 16 threads owns an overlapping tile: thread (tx, ty) sits on
// voxel (x0 - 1 + tx, y0 - 1 + ty) of every plane, and the CTA writes P^k for
// the inner 30 x 14 voxels (tx in 1..30, ty in 1..14).  Walking a chunk of up
// to 64 planes along z, each thread, per plane k:
//   1. forms R = P^{k-1} + c (P^{k-1} - P^{k-2}) at its voxel from registers
//      loaded one plane earlier, and immediately issues the loads of plane
//      k+1 (one plane of loads is always in flight);
//   2. forms U_k = f - lambda div_b R at its voxel: the backward x/y
//      neighbours of R come from shared memory, the backward z neighbour
//      R3(k-1) from its own register (FGP_TV_core.c:220-236, clamp :129);
//   3. one plane behind, forms P^k(k-1) from U's forward differences: x/y
//      from the previous U plane in shared memory, z from the U_k just made
//      (FGP_TV_core.c:237-256), then projects it (utils.c:180-213).
// R and U are formed once per voxel, with 32-bit tile indexing and element
// offsets (below 2^31 voxels), two barriers per plane and no integer division;
// the stopping-check work is compiled only into the check-iteration variant.  Global traffic is the fused
// iteration's 40 B/voxel; the one-voxel halo ring (15% of the tile) is re-read
// from L2.
#include "fgp_tiled.cuh"

#include <stdlib.h>
#include <string.h>

namespace cilreg {

namespace {

constexpr int BX = 32, BY = 16;          // threads
constexpr int OX = BX - 2, OY = BY - 2;  // output voxels per tile
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

struct TiledArgs {
    const float* pc[3];
    const float* po[3];
    float* pn[3];
    const float* f;
    float* u;
    float lam, c, multip;
    int nonneg, aniso, write_u, write_p, check;
    const float* b[3];  // FGP-dTV only: unit gradient field of the reference image
    // momentum from device memory (graph replays): c = carr[*cbase + coff]
    const float* carr;
    const int* cbase;
    int coff;
};

// One tile (bx, by, bz) of one volume: the whole CTA walks its z chunk.
// CHECK: a stopping check (reads U_prev; the caller reduces the returned
// per-thread sums).  IT: element-offset type (int below 2^31 voxels).
// DTV: the FGP-dTV iteration (FGP_dTV_core.c:92-120): R and the gradient of U
// are projected onto the orthogonal complement of a.b at each voxel
// (ProjectVect_func, Grad_dfunc: FGP_dTV_core.c:302-363).
// Loads of state the same kernel may have written: through L2 only (the SM's
// L1 is not coherent with other SMs' stores) in the persistent kernel, which
// runs every iteration in one launch; the read-only path otherwise.
template <bool COHERENT>
__device__ __forceinline__ float ld_state(const float* p) {
    if constexpr (COHERENT) return __ldcg(p);
    else return __ldg(p);
}

template <bool THREE, bool CHECK, typename IT, bool DTV = false, bool COHERENT = false>
__device__ __forceinline__ void fgp_stream_tile(const TiledArgs& a, const Dims& d, int zc, int bx, int by, int bz,
                                                float& pa_out, float& pb_out) {
    __shared__ float sR1[BY][BX];
    __shared__ float sR2[BY][BX];
    __shared__ float sU[2][BY][BX];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = bx * OX + tx - 1;
    const int y = by * OY + ty - 1;
    const int z0 = bz * zc;
    const int z1 = min(z0 + zc, nz);
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool u_pt = in_xy && tx >= 1 && ty >= 1;                    // U needed here
    const bool p_pt = u_pt && tx <= OX && ty <= OY;                    // P written here
    const IT col = in_xy ? ((IT)y * nx + x) : 0;
    const IT sxy = (IT)d.sxy;

    // prefetch registers for one plane
    float c1 = 0.f, o1 = 0.f, c2 = 0.f, o2 = 0.f, c3 = 0.f, o3 = 0.f, fv = 0.f;
    float e1 = 0.f, e2 = 0.f, e3 = 0.f;  // dTV: unit gradient of the reference
    auto load_plane = [&](int k) {
        if (in_xy && k >= 0 && k < nz) {
            const IT v = (IT)k * sxy + col;
            c1 = ld_state<COHERENT>(a.pc[0] + v);
            o1 = ld_state<COHERENT>(a.po[0] + v);
            c2 = ld_state<COHERENT>(a.pc[1] + v);
            o2 = ld_state<COHERENT>(a.po[1] + v);
            if (THREE) {
                c3 = ld_state<COHERENT>(a.pc[2] + v);
                o3 = ld_state<COHERENT>(a.po[2] + v);
            }
            fv = __ldg(a.f + v);
            if (DTV) {
                e1 = __ldg(a.b[0] + v);
                e2 = __ldg(a.b[1] + v);
                if (THREE) e3 = __ldg(a.b[2] + v);
            }
        } else {
            c1 = o1 = c2 = o2 = c3 = o3 = fv = 0.f;
            e1 = e2 = e3 = 0.f;
        }
    };

    float r1p = 0.f, r2p = 0.f, r3p = 0.f, up = 0.f;  // R and U of plane k-1 at this voxel
    float b1p = 0.f, b2p = 0.f, b3p = 0.f;            // dTV: unit gradient of plane k-1
    float uo = 0.f;  // U_prev of the plane the next P step writes (stopping checks only)
    float pa = 0.f, pb = 0.f;
    const float cm = a.carr ? a.carr[*a.cbase + a.coff] : a.c;
    load_plane(z0 - 1);
    for (int k = z0 - 1; k <= z1; ++k) {
        // 1. R of plane k from the prefetched values; start loading plane k+1
        float r1 = c1 + cm * (c1 - o1);
        float r2 = c2 + cm * (c2 - o2);
        float r3 = THREE ? (c3 + cm * (c3 - o3)) : 0.f;
        const float fk = fv;
        const float b1 = e1, b2 = e2, b3 = e3;
        if (DTV) {
            // R onto the complement of the reference's unit gradient (FGP_dTV_core.c:311-314)
            const float ip = THREE ? (r1 * b1 + r2 * b2 + r3 * b3) : (r1 * b1 + r2 * b2);
            r1 = r1 - ip * b1;
            r2 = r2 - ip * b2;
            if (THREE) r3 = r3 - ip * b3;
        }
        if (k < z1) load_plane(k + 1);
        // U_prev of plane k, consumed one plane later: loaded here so that its
        // latency overlaps the barriers instead of stalling the P step
        float uo_next = 0.f;
        if (CHECK && p_pt && k >= z0 && k < z1) {
            if constexpr (COHERENT) uo_next = __ldcg(a.u + (IT)k * sxy + col);
            else uo_next = a.u[(IT)k * sxy + col];
        }
        sR1[ty][tx] = r1;
        sR2[ty][tx] = r2;
        __syncthreads();
        // 2. U of plane k
        float u = 0.f;
        if (u_pt && k >= z0 && k < nz) {
            float s;
            if (THREE)
                s = r1 + r2 + r3 - sR1[ty][tx - 1] - sR2[ty - 1][tx] - r3p;
            else
                s = r1 + r2 - sR1[ty][tx - 1] - sR2[ty - 1][tx];
            u = fk - a.lam * s;
            if (a.nonneg && u < 0.f) u = 0.f;
        }
        sU[k & 1][ty][tx] = u;
        __syncthreads();
        // 3. P^k of plane k-1
        const int kp = k - 1;
        if (p_pt && kp >= z0) {
            const IT v = (IT)kp * sxy + col;
            if (CHECK) {
                const float df = up - uo;
                pa += df * df;
                pb += up * up;
            }
            if (a.write_u) a.u[v] = up;
            if (a.write_p) {
                const int ps = kp & 1;
                float g1 = (x == nx - 1) ? 0.f : up - sU[ps][ty][tx + 1];
                float g2 = (y == ny - 1) ? 0.f : up - sU[ps][ty + 1][tx];
                float g3 = (THREE && kp != nz - 1) ? up - u : 0.f;
                if (DTV) {
                    // gradient onto the complement of the unit gradient (FGP_dTV_core.c:350-356)
                    const float ip = THREE ? (g1 * b1p + g2 * b2p + g3 * b3p) : (g1 * b1p + g2 * b2p);
                    g1 = g1 - ip * b1p;
                    g2 = g2 - ip * b2p;
                    if (THREE) g3 = g3 - ip * b3p;
                }
                float p1 = r1p + a.multip * g1;
                float p2 = r2p + a.multip * g2;
                float p3 = 0.f;
                if (THREE) p3 = r3p + a.multip * g3;
                if (!a.aniso) {
                    const float den = THREE ? (p1 * p1 + p2 * p2 + p3 * p3) : (p1 * p1 + p2 * p2);
                    const float sq = (den > 1.f) ? rsqrtf(den) : 1.f;  // within 2 ulp of 1/sqrtf
                    p1 = p1 * sq;
                    p2 = p2 * sq;
                    p3 = p3 * sq;
                } else {
                    p1 = unit_clip(p1);
                    p2 = unit_clip(p2);
                    p3 = unit_clip(p3);
                }
                a.pn[0][v] = p1;
                a.pn[1][v] = p2;
                if (THREE) a.pn[2][v] = p3;
            }
        }
        r1p = r1;
        r2p = r2;
        r3p = r3;
        if (DTV) {
            b1p = b1;
            b2p = b2;
            b3p = b3;
        }
        up = u;
        uo = uo_next;
    }
    pa_out = pa;
    pb_out = pb;
}

template <bool THREE, bool CHECK, typename IT, bool DTV = false>
__global__ void __launch_bounds__(NT, DTV ? 2 : 3) k_fgp_stream(TiledArgs a, Dims d, int zc, const StopCtl* ctl,
                                                                double2* partials) {
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    if (ctl->stop) return;
    float pa = 0.f, pb = 0.f;
    fgp_stream_tile<THREE, CHECK, IT, DTV>(a, d, zc, blockIdx.x, blockIdx.y, blockIdx.z, pa, pb);
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

template <bool THREE, bool CHECK, typename IT>
__global__ void __launch_bounds__(NT, 3) k_fgp_stream_batch(const FgpBatchVol* __restrict__ vols,
                                                            const int* __restrict__ tile_vol, int it, float c,
                                                            int nonneg, int aniso, int write_u, int write_p) {
    const long long t = blockIdx.x;
    const FgpBatchVol& V = vols[tile_vol[t]];
    if (V.ctl->stop) return;
    const long long lt = t - V.tile_base;
    const int bx = (int)(lt % V.gx);
    const int by = (int)((lt / V.gx) % V.gy);
    const int bz = (int)(lt / ((long long)V.gx * V.gy));
    TiledArgs a;
    for (int q = 0; q < 3; q++) {
        a.pn[q] = V.ring[it % 3][q];
        a.pc[q] = V.ring[(it + 2) % 3][q];
        a.po[q] = V.ring[(it + 1) % 3][q];
    }
    a.f = V.f;
    a.u = V.u;
    a.lam = V.lam;
    a.c = c;
    a.multip = V.multip;
    a.nonneg = nonneg;
    a.aniso = aniso;
    a.write_u = write_u;
    a.write_p = write_p;
    a.check = CHECK;
    a.b[0] = a.b[1] = a.b[2] = nullptr;
    a.carr = nullptr;
    a.cbase = nullptr;
    a.coff = 0;
    float pa = 0.f, pb = 0.f;
    fgp_stream_tile<THREE, CHECK, IT>(a, V.d, V.zc, bx, by, bz, pa, pb);
    if (CHECK) block_pair_partial<NT>(pa, pb, V.partials, lt);
}

// --------------------------------------------------------------------------
// Persistent batched FGP: every iteration of every volume in one launch.
//
// Work items are (iteration, tile) pairs of a group of volumes, handed out by
// an atomic counter in iteration-major order within each group, groups one
// after another.  An item of iteration `it` waits until its volume's
// iteration it-1 is released, i.e. all that volume's tiles of it-1 have
// finished and, on a stopping-check iteration, the volume's check has run.
// Every dependency of an item was handed out before it, to a CTA that is
// running, so the waits always end (no co-residency of the grid is needed).
// A wait still gives up after `wait_limit` polls, sets *error and leaves; the
// host then fails the call.  The last tile to finish an iteration of a volume
// runs that volume's stopping check (the same fixed-order FP64 reduction as
// the finalize kernel) and releases the iteration.  State written within the
// launch is read through L2 (ld.global.cg), never from a stale L1 line.

// one volume's stopping check by the whole CTA (NT = 512 threads): the sums of
// k_finalize_batch's 1024-thread order (thread t and t + 512 of that kernel
// are this thread's two chains), so the relative change is bit-identical
__device__ __forceinline__ void persistent_check(const FgpBatchVol& V, long long ntiles, float epsil, int it) {
    const int tid = threadIdx.x + BX * threadIdx.y;
    double a0 = 0.0, b0 = 0.0, a1 = 0.0, b1 = 0.0;
    for (long long p = tid; p < ntiles; p += 1024) {
        const double2 w = __ldcg(V.partials + p);
        a0 += w.x;
        b0 += w.y;
    }
    for (long long p = tid + 512; p < ntiles; p += 1024) {
        const double2 w = __ldcg(V.partials + p);
        a1 += w.x;
        b1 += w.y;
    }
    __shared__ double sa[32], sb[32];
    a0 = warp_sum(a0);
    b0 = warp_sum(b0);
    a1 = warp_sum(a1);
    b1 = warp_sum(b1);
    if ((tid & 31) == 0) {
        sa[tid >> 5] = a0;
        sb[tid >> 5] = b0;
        sa[16 + (tid >> 5)] = a1;
        sb[16 + (tid >> 5)] = b1;
    }
    __syncthreads();
    if (tid < 32) {
        const double a = warp_sum(sa[tid]);
        const double b = warp_sum(sb[tid]);
        if (tid == 0) {
            StopCtl* c = V.ctl;
            const float re = sqrtf((float)a) / sqrtf((float)b);
            c->re = re;
            if (re < epsil) c->count += 1;
            if (c->count > 3) {
                c->stop = 1;
                c->iters = it;
            }
        }
    }
}

template <bool THREE, typename IT>
__global__ void __launch_bounds__(NT, 3) k_fgp_persistent(FgpPersistArgs A) {
    __shared__ long long s_item;
    __shared__ int s_flag, s_stop;
    const int tid = threadIdx.x + BX * threadIdx.y;
    const long long total = A.gitem[A.ngroups];
    for (;;) {
        if (tid == 0) s_item = (long long)atomicAdd(A.next, 1ULL);
        __syncthreads();
        const long long i = s_item;
        if (i >= total) break;
        int lo = 0, hi = A.ngroups - 1;  // the group holding item i
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (A.gitem[mid] <= i) lo = mid;
            else hi = mid - 1;
        }
        const long long gt0 = A.gtile[lo], nt_group = A.gtile[lo + 1] - gt0;
        const long long r = i - A.gitem[lo];
        const int it = A.it0 + (int)(r / nt_group);
        const long long t = gt0 + r % nt_group;
        const int v = A.tile_vol[t];
        const FgpBatchVol& V = A.vols[v];
        const long long ntv = (long long)V.gx * V.gy * V.gz;
        if (tid == 0) {
            int fl = 0;
            long long polls = 0;
            while (ld_acquire_gpu(A.release + v) < it) {
                if (ld_acquire_gpu(A.error) != 0 || ++polls > A.wait_limit) {
                    atomicExch(A.error, 1);
                    fl = 1;
                    break;
                }
                __nanosleep(200);
            }
            s_flag = fl;
            // read once, after the release: the flag of a check iteration
            // before `it` is final by then
            s_stop = fl ? 0 : ld_acquire_gpu(&V.ctl->stop);
        }
        __syncthreads();
        if (s_flag) break;  // a wait gave up (or another CTA's did): leave, the host reports it
        const bool stopped = s_stop != 0;
        const int check = (A.checking && it % 5 == 0) ? 1 : 0;
        const long long lt = t - V.tile_base;
        if (!stopped) {
            TiledArgs a;
            for (int q = 0; q < 3; q++) {
                a.pn[q] = V.ring[it % 3][q];
                a.pc[q] = V.ring[(it + 2) % 3][q];
                a.po[q] = V.ring[(it + 1) % 3][q];
            }
            a.f = V.f;
            a.u = V.u;
            a.lam = V.lam;
            a.c = A.carr[it];
            a.multip = V.multip;
            a.nonneg = A.nonneg;
            a.aniso = A.aniso;
            a.write_u = (it == A.iters - 1) || check || (A.checking && (it + 1) % 5 == 0);
            a.write_p = (it != A.iters - 1);
            a.check = check;
            a.b[0] = a.b[1] = a.b[2] = nullptr;
            a.carr = nullptr;
            a.cbase = nullptr;
            a.coff = 0;
            const int bx = (int)(lt % V.gx);
            const int by = (int)((lt / V.gx) % V.gy);
            const int bz = (int)(lt / ((long long)V.gx * V.gy));
            float pa = 0.f, pb = 0.f;
            if (check) {
                fgp_stream_tile<THREE, true, IT, false, true>(a, V.d, V.zc, bx, by, bz, pa, pb);
                block_pair_partial<NT>(pa, pb, V.partials, lt);
            } else {
                fgp_stream_tile<THREE, false, IT, false, true>(a, V.d, V.zc, bx, by, bz, pa, pb);
            }
        }
        __syncthreads();  // the tile's stores are issued and its shared memory is free
        if (tid == 0) {
            __threadfence();
            const unsigned long long done = atomicAdd(A.arrive + v, 1ULL) + 1ULL;
            __threadfence();
            s_flag = (done == (unsigned long long)ntv * (unsigned long long)(it - A.it0 + 1)) ? 1 : 0;
        }
        __syncthreads();
        if (s_flag) {  // the last tile of iteration `it` of volume v
            if (check && !stopped) persistent_check(V, ntv, A.epsil, it);
            __syncthreads();
            if (tid == 0) {
                __threadfence();
                st_release_gpu(A.release + v, it + 1);
            }
        }
        __syncthreads();
    }
}

}  // namespace

int fgp_persistent_launch(const FgpPersistArgs& A, bool three, bool wide, int nctas, cudaStream_t s) {
    if (nctas < 1) return fail(ERR_ARG, __FILE__, __LINE__, "no CTAs for the persistent batch");
    const dim3 block(BX, BY, 1);
    decltype(&k_fgp_persistent<true, int>) kern;
    if (!wide) kern = three ? k_fgp_persistent<true, int> : k_fgp_persistent<false, int>;
    else kern = three ? k_fgp_persistent<true, long long> : k_fgp_persistent<false, long long>;
    kern<<<nctas, block, 0, s>>>(A);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

int fgp_persistent_ctas() {
    static const int resident = resident_ctas(k_fgp_persistent<true, int>, NT);
    return sm_count() * resident;
}

void fgp_tile_grid(const Dims& d, int zc, int& gx, int& gy, int& gz) {
    gx = (d.nx + OX - 1) / OX;
    gy = (d.ny + OY - 1) / OY;
    gz = (d.nz + zc - 1) / zc;
}

int fgp_batch_step(const FgpBatchVol* d_vols, const int* d_tile_vol, long long ntiles, bool three, bool wide, int it,
                   float c, int nonneg, int aniso, int write_u, int write_p, int check, cudaStream_t s) {
    if (ntiles < 1 || ntiles > 2147483647LL) return fail(ERR_ARG, __FILE__, __LINE__, "tile count %lld", ntiles);
    const dim3 grid((unsigned)ntiles);  // one CTA per tile of every volume
    const dim3 block(BX, BY, 1);
    decltype(&k_fgp_stream_batch<true, true, int>) kern;
    if (!wide)
        kern = three ? (check ? k_fgp_stream_batch<true, true, int> : k_fgp_stream_batch<true, false, int>)
                     : (check ? k_fgp_stream_batch<false, true, int> : k_fgp_stream_batch<false, false, int>);
    else
        kern = three ? (check ? k_fgp_stream_batch<true, true, long long> : k_fgp_stream_batch<true, false, long long>)
                     : (check ? k_fgp_stream_batch<false, true, long long>
                              : k_fgp_stream_batch<false, false, long long>);
    kern<<<grid, block, 0, s>>>(d_vols, d_tile_vol, it, c, nonneg, aniso, write_u, write_p);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

int fgp_default_zchunk(const Dims& d) { return (d.nz > 1) ? ((d.nz < ZCHUNK) ? d.nz : ZCHUNK) : 1; }

__global__ void k_add_int(int* p, int v) { *p += v; }

int fgp_advance_base(int* base, int by, cudaStream_t s) {
    k_add_int<<<1, 1, 0, s>>>(base, by);
    CILREG_CUDA(cudaGetLastError());
    note_launch();
    return OK;
}

TiledPlan fgp_tiled_plan(const Dims& d, int resident_ctas_per_sm) {
    TiledPlan T;
    const char* e = getenv("CILREG_FGP_KERNEL");
    T.use = !(e && strcmp(e, "simple") == 0);  // "simple" selects the per-voxel kernel of fgp.cu
    T.block = dim3(BX, BY, 1);
    if (d.nz > 1) {
        // one volume: balance the CTAs over the SMs (the batched path packs
        // many volumes and keeps fgp_default_zchunk)
        static const int resident = resident_ctas(k_fgp_stream<true, false, int>, NT);
        const long long tiles = (long long)((d.nx + OX - 1) / OX) * ((d.ny + OY - 1) / OY);
        T.zchunk = wave_zchunk(tiles, d.nz, resident_ctas_per_sm > 0 ? resident_ctas_per_sm : resident, 2, ZCHUNK);
    } else {
        T.zchunk = 1;
    }
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int fgp_tiled_step(const TiledPlan& T, const float* const pc[3], const float* const po[3], float* const pn[3],
                   const float* f, float* u, float lam, float c, float multip, int nonneg, int aniso, int write_u,
                   int write_p, int check, const Dims& d, const StopCtl* ctl, double2* partials, cudaStream_t s,
                   const float* const* b, const float* carr, const int* cbase, int coff) {
    if (T.x2 && (!b || d.nz == 1))
        return fgp_x2_step(T, pc, po, pn, f, u, lam, c, multip, nonneg, aniso, write_u, write_p, check, d, ctl,
                           partials, s, carr, cbase, coff, b);
    TiledArgs a;
    a.carr = carr;
    a.cbase = cbase;
    a.coff = coff;
    for (int i = 0; i < 3; i++) {
        a.pc[i] = pc[i];
        a.po[i] = po[i];
        a.pn[i] = pn[i];
    }
    a.f = f;
    a.u = u;
    a.lam = lam;
    a.c = c;
    a.multip = multip;
    a.nonneg = nonneg;
    a.aniso = aniso;
    a.write_u = write_u;
    a.write_p = write_p;
    a.check = check;
    for (int i = 0; i < 3; i++) a.b[i] = b ? b[i] : nullptr;
    const bool three = d.nz > 1;
    decltype(&k_fgp_stream<true, true, int>) kern;
    if (b) {
        if (d.n < (1LL << 31))
            kern = three ? (check ? k_fgp_stream<true, true, int, true> : k_fgp_stream<true, false, int, true>)
                         : (check ? k_fgp_stream<false, true, int, true> : k_fgp_stream<false, false, int, true>);
        else
            kern = three ? (check ? k_fgp_stream<true, true, long long, true>
                                  : k_fgp_stream<true, false, long long, true>)
                         : (check ? k_fgp_stream<false, true, long long, true>
                                  : k_fgp_stream<false, false, long long, true>);
    } else if (d.n < (1LL << 31))
        kern = three ? (check ? k_fgp_stream<true, true, int> : k_fgp_stream<true, false, int>)
                     : (check ? k_fgp_stream<false, true, int> : k_fgp_stream<false, false, int>);
    else
        kern = three ? (check ? k_fgp_stream<true, true, long long> : k_fgp_stream<true, false, long long>)
                     : (check ? k_fgp_stream<false, true, long long> : k_fgp_stream<false, false, long long>);
    CILREG_CUDA(launch_pdl(kern, T.grid, T.block, 0, s, a, d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg
