// FGP-TV: Beck-Teboulle fast gradient projection on the dual of TV
// (reference: FGP_TV_core.c:40-269, projections utils.c:149-213).
//
// State kept in HBM is only the dual iterates P^{k-1}, P^{k-2} (three ring
// buffers of d components) and the data f.  The reference's R and U arrays
// are never stored:
//   R^{(k)} = P^{k-1} + c_{k-1} (P^{k-1} - P^{k-2}),  c_{k-1} = (t_{k-1}-1)/t_k
//   U_k     = f - lambda * div_b R^{(k)}      (zero flux below index 0)
//   P^k     = proj( R^{(k)} + m (U_k - U_k[+1]) )   (zero at the last index)
// so one kernel per iteration reads P^{k-1}, P^{k-2}, f and writes P^k:
// 40 B per voxel-iteration in 3D (28 B in 2D).  U_k is written to the output
// only on iterations that need it (the last one, stopping checks, and the
// iteration before a check, whose U is the check's U_prev).
#include <vector>

#include "drivers.cuh"
#include "fgp_tiled.cuh"
#include "nvtx.cuh"

namespace cilreg {

namespace {

struct FgpArgs {
    const float* pc[3];  // P^{k-1}
    const float* po[3];  // P^{k-2}
    float* pn[3];        // P^k (output)
    const float* f;
    float* u;            // U output / U_prev of the next check
    float lam, c, multip;
    int nonneg, aniso, write_u, write_p, check;
};

template <bool THREE>
__device__ __forceinline__ float r_at(const FgpArgs& a, int comp, long long v) {
    const float p = ldg(a.pc[comp], v);
    return p + a.c * (p - ldg(a.po[comp], v));
}

// U at (i,j,k) from R (FGP_TV_core.c:220-236), then the optional clamp (:129)
template <bool THREE>
__device__ __forceinline__ float u_at(const FgpArgs& a, const Dims& d, int i, int j, int k) {
    const long long v = vid(d, i, j, k);
    const float b1 = (i == 0) ? 0.0f : r_at<THREE>(a, 0, v - 1);
    const float b2 = (j == 0) ? 0.0f : r_at<THREE>(a, 1, v - d.nx);
    float u;
    if (THREE) {
        const float b3 = (k == 0) ? 0.0f : r_at<THREE>(a, 2, v - d.sxy);
        u = ldg(a.f, v) - a.lam * (r_at<THREE>(a, 0, v) + r_at<THREE>(a, 1, v) + r_at<THREE>(a, 2, v) - b1 - b2 - b3);
    } else {
        u = ldg(a.f, v) - a.lam * (r_at<THREE>(a, 0, v) + r_at<THREE>(a, 1, v) - b1 - b2);
    }
    if (a.nonneg && u < 0.0f) u = 0.0f;
    return u;
}

template <bool THREE>
__global__ void __launch_bounds__(256) k_fgp_step(FgpArgs a, Dims d, int kz, const StopCtl* ctl,
                                                  double2* partials) {
    if (ctl->stop) return;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k0 = blockIdx.z * kz;
    float pa = 0.0f, pb = 0.0f;
    if (i < d.nx && j < d.ny) {
        for (int kk = 0; kk < kz; kk++) {
            const int k = k0 + kk;
            if (k >= d.nz) break;
            const long long v = vid(d, i, j, k);
            const float u = u_at<THREE>(a, d, i, j, k);
            if (a.check) {
                const float df = u - a.u[v];
                pa += df * df;
                pb += u * u;
            }
            if (a.write_u) a.u[v] = u;
            if (a.write_p) {
                // gradient step (FGP_TV_core.c:237-256)
                const float g1 = (i == d.nx - 1) ? 0.0f : u - u_at<THREE>(a, d, i + 1, j, k);
                const float g2 = (j == d.ny - 1) ? 0.0f : u - u_at<THREE>(a, d, i, j + 1, k);
                float p1 = r_at<THREE>(a, 0, v) + a.multip * g1;
                float p2 = r_at<THREE>(a, 1, v) + a.multip * g2;
                float p3 = 0.0f;
                if (THREE) {
                    const float g3 = (k == d.nz - 1) ? 0.0f : u - u_at<THREE>(a, d, i, j, k + 1);
                    p3 = r_at<THREE>(a, 2, v) + a.multip * g3;
                }
                // projection (utils.c:180-213)
                if (!a.aniso) {
                    const float den = THREE ? (p1 * p1 + p2 * p2 + p3 * p3) : (p1 * p1 + p2 * p2);
                    if (den > 1.0f) {
                        const float sq = rsqrtf(den);  // within 2 ulp of 1/sqrtf
                        p1 = p1 * sq;
                        p2 = p2 * sq;
                        p3 = p3 * sq;
                    }
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
    }
    if (a.check) block_pair_partial<256>(pa, pb, partials, block_slot());
}

}  // namespace

int fgp_run(const float* f, float* u_out, float lam, int iters, float epsil, int methodTV, int nonneg,
            const Dims& d, cudaStream_t s, float* info, FgpWarm* warm) {
    CILREG_RANGE("cilreg FGP-TV");
    const bool three = d.nz > 1;
    const int nc = three ? 3 : 2;
    Scratch scratch(s);
    const Launch3 L = plan_launch(d);
    TiledPlan T = fgp_tiled_plan(d);
    // P^j lives in ring[j mod R]: R = 3 for single iterations (P^k overwrites
    // P^{k-3}); R = 4 when iterations run in pairs, whose second output P^{k+1}
    // must not overwrite the P^{k-2} that neighbouring tiles still read
    const PairPlan TP = (T.use && !warm) ? fgp_pair_plan(d) : PairPlan{};
    const int R = TP.use ? 4 : 3;
    // the tensor-copy kernel: same tiles, z chunks balanced for its own occupancy
    bool tma = T.use && !TP.use && fgp_tma_usable(d);
    if (tma) {
        T = fgp_tiled_plan(d, fgp_tma_resident());
    } else if (T.use && !TP.use) {
        // below the tensor-copy kernel's sizes: two voxels per thread
        const TiledPlan X = fgp_x2_plan(d);
        if (X.use) T = X;
    }
    IterControl ctl(s, scratch, iters, epsil, T.use ? T.nblocks : num_blocks(L));
    CILREG_TRY(ctl.status());
    float* ring[4][3] = {};
    int base = 0;
    if (warm) {
        // warm start: the caller's dual buffers hold P_{-1}, P_{-2} of this call
        base = warm->base;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) ring[r][c] = warm->ring[(base + r) % 3][c];
    } else {
        for (int r = 0; r < R; r++)
            for (int c = 0; c < nc; c++) {
                ring[r][c] = scratch.floats(d.n);
                if (!ring[r][c]) return scratch.status();
            }
        // P^{-1} = P^{-2} = 0 (the reference's calloc'd P, P_prev, R)
        for (int r = R - 2; r < R; r++)
            for (int c = 0; c < nc; c++) CILREG_CUDA(cudaMemsetAsync(ring[r][c], 0, sizeof(float) * d.n, s));
    }

    // tensor maps of (P^{k-1}, P^{k-2}, f) for each position of the ring
    std::vector<unsigned char> maps;
    if (tma) {
        const size_t mb = fgp_tma_maps_bytes();
        maps.resize(mb * R);
        for (int r = 0; r < R && tma; r++) {
            const float* arr[7] = {ring[(r + R - 1) % R][0], ring[(r + R - 1) % R][1], ring[(r + R - 1) % R][2],
                                   ring[(r + R - 2) % R][0], ring[(r + R - 2) % R][1], ring[(r + R - 2) % R][2],
                                   f};
            tma = fgp_tma_encode(arr, d, maps.data() + mb * r);
        }
    }

    const float multip = three ? (1.0f / (12.0f * lam)) : (1.0f / (8.0f * lam));
    float tk = 1.0f;   // t_{k}
    float cprev = 0.0f;  // c_{k-1}; R^{(0)} = 0 whatever its value
    auto writes_u = [&](int k) {
        return (k == iters - 1) || ctl.is_check(k) || (ctl.checking() && ((k + 1) % 5 == 0));
    };
    auto writes_p = [&](int k) { return (k != iters - 1) || warm != nullptr; };
    int it = 0;
    constexpr int G = 66;  // replayed block: a multiple of the ring's period 3, even
    if (T.use && !tma && !TP.use && !ctl.checking() && d.n <= (1LL << 22) && iters > 2 * G) {
        // small volume, fixed count: iterations 0 .. iters-2 from a replayed
        // graph, their momentum coefficients read on the device from the
        // sequence formed here (FGP_TV_core.c:138-139); the last one directly
        std::vector<float> cseq(iters);
        for (int k = 0; k < iters; k++) {
            cseq[k] = cprev;
            const float tkp1 = (1.0f + sqrtf(1.0f + 4.0f * tk * tk)) * 0.5f;
            cprev = (tk - 1.0f) / tkp1;
            tk = tkp1;
        }
        float* carr = scratch.floats(iters);
        int* cbase = (int*)scratch.bytes(sizeof(int));
        if (!carr || !cbase) return scratch.status();
        CILREG_CUDA(cudaMemcpyAsync(carr, cseq.data(), sizeof(float) * iters, cudaMemcpyHostToDevice, s));
        CILREG_CUDA(cudaMemsetAsync(cbase, 0, sizeof(int), s));
        auto iteration = [&](int k, cudaStream_t st, bool in_graph) -> int {
            float* pn[3] = {ring[k % R][0], ring[k % R][1], ring[k % R][2]};
            const float* pc[3] = {ring[(k + R - 1) % R][0], ring[(k + R - 1) % R][1], ring[(k + R - 1) % R][2]};
            const float* po[3] = {ring[(k + R - 2) % R][0], ring[(k + R - 2) % R][1], ring[(k + R - 2) % R][2]};
            CILREG_TRY(fgp_tiled_step(T, pc, po, pn, f, u_out, lam, cseq[k], multip, nonneg == 1, methodTV != 0,
                                      writes_u(k) ? 1 : 0, writes_p(k) ? 1 : 0, 0, d, ctl.ctl(), nullptr, st, nullptr,
                                      in_graph ? carr : nullptr, cbase, k));
            note_launch();
            return OK;
        };
        CILREG_TRY(run_replayed(iters - 1, G, s, iteration,
                                [&](cudaStream_t st) -> int { return fgp_advance_base(cbase, G, st); }));
        CILREG_TRY(iteration(iters - 1, s, false));
        it = iters;
    }
    for (; it < iters; it++) {
        const int check = ctl.is_check(it) ? 1 : 0;
        if (TP.use && it + 1 < iters && !check && !ctl.is_check(it + 1) && !writes_u(it) && writes_p(it)) {
            // iterations it and it+1 in one pass
            const float tkp1 = (1.0f + sqrtf(1.0f + 4.0f * tk * tk)) * 0.5f;
            const float cnext = (tk - 1.0f) / tkp1;
            float* pn1[3] = {ring[it % R][0], ring[it % R][1], ring[it % R][2]};
            float* pn2[3] = {ring[(it + 1) % R][0], ring[(it + 1) % R][1], ring[(it + 1) % R][2]};
            const float* pc[3] = {ring[(it + R - 1) % R][0], ring[(it + R - 1) % R][1], ring[(it + R - 1) % R][2]};
            const float* po[3] = {ring[(it + R - 2) % R][0], ring[(it + R - 2) % R][1], ring[(it + R - 2) % R][2]};
            CILREG_TRY(fgp_pair_step(TP, pc, po, pn1, pn2, f, u_out, lam, cprev, cnext, multip, nonneg == 1,
                                     methodTV != 0, writes_u(it + 1) ? 1 : 0, writes_p(it + 1) ? 1 : 0, d, ctl.ctl(),
                                     s));
            note_launch();
            // advance the momentum sequence by two iterations (FGP_TV_core.c:138-139)
            tk = tkp1;
            cprev = cnext;
            const float tkp2 = (1.0f + sqrtf(1.0f + 4.0f * tk * tk)) * 0.5f;
            cprev = (tk - 1.0f) / tkp2;
            tk = tkp2;
            it++;
            continue;
        }
        FgpArgs a;
        for (int c = 0; c < 3; c++) {
            a.pn[c] = ring[it % R][c];
            a.pc[c] = ring[(it + R - 1) % R][c];
            a.po[c] = ring[(it + R - 2) % R][c];
        }
        a.f = f;
        a.u = u_out;
        a.lam = lam;
        a.c = cprev;
        a.multip = multip;
        a.nonneg = (nonneg == 1);
        a.aniso = (methodTV != 0);
        a.check = check;
        a.write_u = writes_u(it);
        a.write_p = writes_p(it);  // a warm state keeps the last dual iterate
        if (tma)
            CILREG_TRY(fgp_tma_step(T, maps.data() + fgp_tma_maps_bytes() * (it % R), a.pn, u_out, lam, cprev, multip,
                                    a.nonneg, a.aniso, a.write_u, a.write_p, check, d, ctl.ctl(), ctl.partials(), s));
        else if (T.use)
            CILREG_TRY(fgp_tiled_step(T, a.pc, a.po, a.pn, f, u_out, lam, cprev, multip, a.nonneg, a.aniso,
                                      a.write_u, a.write_p, check, d, ctl.ctl(), ctl.partials(), s));
        else if (three)
            k_fgp_step<true><<<L.grid, L.block, 0, s>>>(a, d, L.kz, ctl.ctl(), ctl.partials());
        else
            k_fgp_step<false><<<L.grid, L.block, 0, s>>>(a, d, L.kz, ctl.ctl(), ctl.partials());
        CILREG_CUDA(cudaGetLastError());
        note_launch();
        // t_{k+1} and the momentum coefficient for the next R (FGP_TV_core.c:138-139)
        const float tkp1 = (1.0f + sqrtf(1.0f + 4.0f * tk * tk)) * 0.5f;
        cprev = (tk - 1.0f) / tkp1;
        tk = tkp1;
        if (check) {
            CILREG_TRY(ctl.after_check(it, T.use ? T.nblocks : num_blocks(L)));
            if (ctl.host_should_stop()) break;
        }
    }
    StopCtl done;
    CILREG_TRY(ctl.finish(info, &done));
    if (tma) CILREG_TRY(fgp_tma_status(s));
    if (warm) {
        // iterations 0..last wrote ring[(base + it) % 3]
        const int ran = done.stop ? done.iters + 1 : iters;
        warm->base = (base + ran) % 3;
    }
    return OK;
}

}  // namespace cilreg
