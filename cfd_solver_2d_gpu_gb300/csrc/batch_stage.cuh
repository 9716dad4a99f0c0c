// The batched persistent stage kernel (one cooperative launch per Runge-Kutta
// stage) and its instantiation helpers; see batch.cu for the design.
#pragma once
#include <cuda_runtime.h>

#include "step_device.cuh"

namespace fvgb {
namespace dev {

struct InstState {
    double t, T, dt, dt6, dt_raw, CFL;
    unsigned long long dtmin_bits;
    double t_old;  // t at the start of the step (the clock of the double-Mach-reflection boundary)
};

struct GridBarrier {
    unsigned int count;
    unsigned int gen;
    unsigned int error;      // 1 = a barrier wait gave up
    unsigned int queue[16];  // work-queue counters of the dynamic schedule, one per phase
};

struct BatchView {
    MeshView m;                  // packed mesh (global indices)
    int n_inst;
    const int* __restrict__ c_inst;   // instance of each cell
    const int* __restrict__ e_inst;   // instance of each edge
    const BcData* __restrict__ bc;    // per instance
    InstState* inst;
    const int* __restrict__ cell_key;     // reference order across the batch (instance, then reference index)
    const int* __restrict__ dev_of_key;
    d4 *U, *U0, *K1, *Gx, *Gy, *F, *prim, *rhs;
    double *alpha, *alpha_vis;
    int* flags;
    unsigned int* flag_count;
    int flag_cap;
    Status* status;
    GridBarrier* bar;
    int tile;        // items per work tile (a multiple of the block size)
    int dynamic;     // 1: tiles taken from an atomic work queue; 0: static round-robin
    int restrict_ref;
    double value_1;
};

constexpr long long kBarrierSpinLimit = 20000000;  // ~0.6 s of 32 ns sleeps, far above any phase here

// bounded sense-reversal barrier over all blocks of a cooperative launch: a block that
// waits more than `limit` polls (or sees another's give-up) sets the error word and
// returns false, so a missing block ends the kernel instead of hanging it
__device__ __forceinline__ bool grid_sync(GridBarrier* b, long long limit = kBarrierSpinLimit) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned int* vgen = &b->gen;
        const unsigned int g = *vgen;
        __threadfence();
        const unsigned int arrived = atomicAdd(&b->count, 1u);
        if (arrived == gridDim.x - 1) {
            b->count = 0;
            __threadfence();
            atomicAdd(&b->gen, 1u);
        } else {
            long long it = 0;
            while (*vgen == g) {
                if (++it > limit || *(volatile unsigned int*)&b->error) {
                    atomicExch(&b->error, 1u);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        if (*(volatile unsigned int*)&b->error) ok = 0;
    }
    __syncthreads();
    return ok != 0;
}

// visits items [0, n) in tiles of bv.tile, statically or from the work queue of `phase`
template <class F>
__device__ __forceinline__ void for_tiles(const BatchView& bv, int n, int phase, F&& body) {
    const int ntiles = (n + bv.tile - 1) / bv.tile;
    if (bv.dynamic) {
        __shared__ int t_sh;
        while (true) {
            if (threadIdx.x == 0) t_sh = (int)atomicAdd(&bv.bar->queue[phase], 1u);
            __syncthreads();
            const int t = t_sh;
            __syncthreads();
            if (t >= ntiles) break;
            const int end = min(n, (t + 1) * bv.tile);
            for (int i = t * bv.tile + threadIdx.x; i < end; i += blockDim.x) body(i);
        }
    } else {
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            const int end = min(n, (t + 1) * bv.tile);
            for (int i = t * bv.tile + threadIdx.x; i < end; i += blockDim.x) body(i);
        }
    }
}

template <int KIND, int FLUX, bool LINEAR, bool GRADIENT, int GRAD, bool BARTH, bool NS>
__global__ void k_batch_stage(BatchView bv, Gas g) {
    const MeshView& m = bv.m;
    constexpr bool FIRST = (KIND == STAGE_EULER || KIND == STAGE_RK3_1 || KIND == STAGE_SSP_1);
    // reset the work queues of the phases this launch uses (the previous launch finished them)
    if (bv.dynamic) {
        if (blockIdx.x == 0 && threadIdx.x < 16) bv.bar->queue[threadIdx.x] = 0;
        if (!grid_sync(bv.bar)) return;
    }
    if (FIRST) {
        const bool copy = KIND != STAGE_EULER;
        for_tiles(bv, m.N, 0, [&](int c) { prim_cell(c, bv.U, bv.U0, bv.prim, g, copy); });
        if (!grid_sync(bv.bar)) return;
        for_tiles(bv, m.E, 1, [&](int e) { alpha_edge<NS>(e, bv.prim, m, g, bv.value_1, bv.alpha, bv.alpha_vis, bv.status); });
        if (!grid_sync(bv.bar)) return;
        // per-instance minimum: segmented warp reduction over contiguous cells of one instance
        const int ntiles = (m.N + bv.tile - 1) / bv.tile;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            const int end = min(m.N, (t + 1) * bv.tile);
            for (int base = t * bv.tile; base < end; base += blockDim.x) {
                const int c = base + threadIdx.x;
                const bool live = c < end;
                const int inst = live ? __ldg(&bv.c_inst[c]) : -1;
                double v = live ? dt_cell<NS>(c, m, bv.alpha, bv.alpha_vis, bv.inst[inst].CFL) : 1e10;
                const int lane = threadIdx.x & 31;
                for (int o = 1; o < 32; o <<= 1) {
                    const double v2 = __shfl_down_sync(0xffffffffu, v, o);
                    const int i2 = __shfl_down_sync(0xffffffffu, inst, o);
                    if (lane + o < 32 && i2 == inst) v = dmin(v, v2);
                }
                const int iprev = __shfl_up_sync(0xffffffffu, inst, 1);
                if (live && (lane == 0 || iprev != inst)) {
                    if (!neg(v) && !is_nan(v)) dmin_atomic(&bv.inst[inst].dtmin_bits, v);
                    else atomicMin(&bv.inst[inst].dtmin_bits, 0ull);
                }
            }
        }
        if (!grid_sync(bv.bar)) return;
        // t clamp per instance (CIteration.cpp:134-139)
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < bv.n_inst; i += gridDim.x * blockDim.x) {
            InstState& s = bv.inst[i];
            double dt = __longlong_as_double((long long)s.dtmin_bits);
            s.dt_raw = dt;
            if (s.t + dt > s.T) dt = s.T - s.t;
            s.t_old = s.t;
            s.t += dt;
            s.dt = dt;
            s.dt6 = dt / 6.0;
            s.dtmin_bits = (unsigned long long)__double_as_longlong(1e10);
        }
        if (!grid_sync(bv.bar)) return;
    }
    if (GRADIENT) {
        for_tiles(bv, m.N, 2, [&](int c) { grad_cell<GRAD, BARTH>(c, bv.U, m, bv.Gx, bv.Gy); });
        if (!grid_sync(bv.bar)) return;
    }
    for_tiles(bv, m.E, 3, [&](int e) {
        if (e < m.E_int) {
            flux_interior<FLUX, LINEAR, NS>(e, bv.U, bv.Gx, bv.Gy, m, g, bv.F);
        } else {
            BcData bc = bv.bc[__ldg(&bv.e_inst[e])];
            bc.clock_frac = dsr_stage_frac(KIND);
            flux_boundary<FLUX, LINEAR, NS>(e, bv.U, bv.Gx, bv.Gy, m, g, bc, bv.F, bv.status);
        }
    });
    if (!grid_sync(bv.bar)) return;
    for_tiles(bv, m.N, 4, [&](int c) {
        const InstState& s = bv.inst[__ldg(&bv.c_inst[c])];
        update_cell<KIND>(c, bv.U, bv.U0, bv.K1, bv.rhs, bv.F, m, s.dt, s.dt6, g, bv.flags, bv.flag_count,
                          bv.flag_cap, bv.status);
    });
    if (final_stage(KIND)) {
        if (!grid_sync(bv.bar)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0)
            restrict_pass(bv.U, m, bv.cell_key, bv.dev_of_key, m.N, bv.flags, bv.flag_count, bv.flag_cap,
                          bv.restrict_ref, g, bv.status);
    }
}

}  // namespace dev

namespace batch_detail {
using StageFn = void (*)(dev::BatchView, dev::Gas);

template <int KIND, int FLUX, bool LINEAR, bool GRADIENT, int GRAD, bool BARTH, bool NS>
inline StageFn stage_ptr() {
    return dev::k_batch_stage<KIND, FLUX, LINEAR, GRADIENT, GRAD, BARTH, NS>;
}

// the gradient variants of one flux: with linear reconstruction, and (Navier-Stokes only) with
// constant reconstruction, whose viscous fluxes still read gradients
template <int KIND, int FLUX, bool NS>
inline StageFn pick_grad(bool linear, int grad, bool barth) {
    if (linear) {
        if (grad == 1) return barth ? stage_ptr<KIND, FLUX, true, true, 1, true, NS>() : stage_ptr<KIND, FLUX, true, true, 1, false, NS>();
        return barth ? stage_ptr<KIND, FLUX, true, true, 2, true, NS>() : stage_ptr<KIND, FLUX, true, true, 2, false, NS>();
    }
    if constexpr (NS) {
        if (grad == 1) return barth ? stage_ptr<KIND, FLUX, false, true, 1, true, NS>() : stage_ptr<KIND, FLUX, false, true, 1, false, NS>();
        return barth ? stage_ptr<KIND, FLUX, false, true, 2, true, NS>() : stage_ptr<KIND, FLUX, false, true, 2, false, NS>();
    } else {
        return stage_ptr<KIND, FLUX, false, false, 1, false, false>();
    }
}

template <int KIND>
inline StageFn pick_kind(int flux, bool linear, int grad, bool barth, bool ns) {
    if (flux == 2002) return ns ? pick_grad<KIND, 2002, true>(linear, grad, barth) : pick_grad<KIND, 2002, false>(linear, grad, barth);
    return ns ? pick_grad<KIND, 2001, true>(linear, grad, barth) : pick_grad<KIND, 2001, false>(linear, grad, barth);
}

}  // namespace batch_detail

using StageFn = batch_detail::StageFn;
// one translation unit per stage kind instantiates its kernels (parallel build)
StageFn batch_stage_euler(int flux, bool linear, int grad, bool barth, bool ns);
StageFn batch_stage_rk3_1(int flux, bool linear, int grad, bool barth, bool ns);
StageFn batch_stage_rk3_2(int flux, bool linear, int grad, bool barth, bool ns);
StageFn batch_stage_rk3_3(int flux, bool linear, int grad, bool barth, bool ns);
StageFn batch_stage_ssp_1(int flux, bool linear, int grad, bool barth, bool ns);
StageFn batch_stage_ssp_2(int flux, bool linear, int grad, bool barth, bool ns);
StageFn batch_stage_ssp_3(int flux, bool linear, int grad, bool barth, bool ns);

}  // namespace fvgb
