// gbo_sim.cuh -- run!(simulation) on the device: the loop of time_step!(sim) with its
// stop criteria, time-step alignment, NaNChecker and TimeStepWizard, so that a whole
// run of many time steps is one CUDA-graph launch with no host round trip.
//
// Reference behaviour restated here:
//   * time_step!(sim): Δt aligned with stop_time, model step, then the callbacks
//     whose schedule actuates (src/Simulations/run.jl:214-262, :37-53);
//   * the callbacks a Simulation registers, in order: stop_time_exceeded,
//     stop_iteration_exceeded, wall_time_limit_exceeded, NaNChecker on the first
//     prognostic field every 100 iterations (simulation.jl:87-94, 243-269;
//     Models/Models.jl:201-212; Diagnostics/nan_checker.jl:48-66), then the
//     TimeStepWizard on IterationInterval(N) (time_step_wizard.jl:97-115);
//   * initialize!(sim) of a fresh simulation evaluates every callback once at
//     iteration 0 (run.jl:319-347);
//   * cell_advection_timescale = min over cells of 1 / (|u|/Δxᶠᶜᶜ + |v|/Δyᶜᶠᶜ + |w|/Δzᶜᶜᶠ)
//     (Advection/cell_advection_timescale.jl:15-36) and the diffusion timescales of
//     Smagorinsky-Lilly and AMD (TurbulenceClosures/turbulence_closure_diagnostics.jl:48-63).
//
// State lives in a small FP64 array (RUN_* slots).  k_sim_begin aligns Δt and writes
// its stage factors (stage_factors), which every stage kernel of the step reads;
// k_sim_callbacks reduces
// the fields when a callback is due (one partial per block, the last block combines
// them), advances the clock, evaluates the callbacks and sets the loop condition.
#pragma once
#include <math_constants.h>

#include "gbo_cg.cuh"

enum {
    RUN_DT = 0,        // Δt of the step being taken (after alignment)
    RUN_SIM_DT,        // simulation.Δt, in the model's float type
    RUN_TIME, RUN_ITER,
    RUN_STOP_TIME,     // in the model's float type (Simulation converts it)
    RUN_STOP_ITER,
    RUN_ALIGN,
    RUN_RUNNING, RUN_REASON, RUN_NAN,
    RUN_TAKEN,         // iterations taken by this launch of the loop
    RUN_MAX_TAKEN,     // iterations one launch may take
    RUN_WIZ_EVERY, RUN_CFL, RUN_DCFL, RUN_MAX_CHANGE, RUN_MIN_CHANGE, RUN_MAX_DT, RUN_MIN_DT,
    RUN_NAN_EVERY,
    RUN_DELTA2,        // Δ² of the diffusion timescale (minimum spacing squared, in FT)
    RUN_PR_FACTOR,     // max(1, 1 / Pr) of Smagorinsky-Lilly, in FT
    RUN_TAU_ADV, RUN_TAU_DIF,  // timescales of the last reduction
    RUN_LAST_DT,       // clock.last_Δt (QAB2 takes an Euler step when Δt differs from it)
    RUN_NSLOTS
};

enum { SIM_INIT = 0, SIM_AFTER_STEP = 1, SIM_TIMESCALES = 2 };
constexpr int SIM_BLOCKS = 2 * 152;
constexpr int SIM_PARTS = 4;  // per block: max 1/τ, max νₑ, max κₑ, NaN found

// Julia's min / max / clamp on floats: a NaN operand gives NaN
GBO_HD double jmin(double a, double b) { return (a != a || b != b) ? a + b : (b < a ? b : a); }
GBO_HD double jmax(double a, double b) { return (a != a || b != b) ? a + b : (b > a ? b : a); }
GBO_HD double jclamp(double x, double lo, double hi) { return x > hi ? hi : (x < lo ? lo : x); }

template <typename FT>
struct SimP {
    GridP<FT> g;
    const FT* u; const FT* v; const FT* w;
    const FT* nu;
    const FT* kap[GBO_MAX_TRACERS];
    int ntr, closure;
    double* run;
    double* part;
    unsigned int* cnt;
};

// c of Δτ = FT(Δt c) for the three RK3 stages
struct StageC {
    double c0, c1, c2;
};

// Stage factors of Δt (stage_factors) for the stage kernels of the next steps
template <typename FT>
__global__ void k_set_dt(FT* dtf, double dt, StageC c) { stage_factors<FT>(dt, c.c0, c.c1, c.c2, dtf); }
// the same for the FP32 and the FP64 members of an ensemble
__global__ void k_set_dt_pair(float* f32, StageC c32, double* f64, StageC c64, double dt) {
    stage_factors<float>(dt, c32.c0, c32.c1, c32.c2, f32);
    stage_factors<double>(dt, c64.c0, c64.c1, c64.c2, f64);
}

// First node of a loop launch: no iterations taken yet.
__global__ void k_sim_start(double* run) { run[RUN_TAKEN] = 0.0; }

// aligned_time_step (run.jl:37-53): Δt = min(simulation.Δt, stop_time - time), and
// simulation.Δt again when that is not positive; its stage factors go to dtf.  Clears
// the loop condition first: only the last block of k_sim_callbacks sets it, so an
// iteration whose callbacks did not run ends the loop instead of repeating it.  With
// QAB2 it selects the Euler branch when Δt differs from clock.last_Δt
// (quasi_adams_bashforth_2.jl:101).
template <typename FT>
__global__ void k_sim_begin(double* run, FT* dtf, StageC c, cudaGraphConditionalHandle h,
                            cudaGraphConditionalHandle h_euler, int use_handle, int qab2) {
    if (use_handle) cudaGraphSetConditional(h, 0u);
    const double dt = run[RUN_SIM_DT];
    double a = dt;
    if (run[RUN_ALIGN] != 0.0) {
        a = jmin(a, run[RUN_STOP_TIME] - run[RUN_TIME]);
        a = a <= 0.0 ? dt : a;
    }
    run[RUN_DT] = a;
    stage_factors<FT>(a, c.c0, c.c1, c.c2, dtf);
    if (use_handle && qab2) cudaGraphSetConditional(h_euler, a != run[RUN_LAST_DT] ? 1u : 0u);
}

GBO_D double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = jmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}
// block maximum (NaN-propagating) of one value per thread; valid in thread 0
GBO_D double block_max(double v, double* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < nw ? sh[lane] : -CUDART_INF;
        v = warp_max(v);
    }
    return v;
}

// new_time_step (time_step_wizard.jl:97-112) with the wizard's parameters in FP64;
// the result is stored into simulation.Δt, whose type is the model's float type.
template <typename FT>
GBO_D double wizard_dt(const double* R, double old_dt) {
    const double adv = R[RUN_CFL] * R[RUN_TAU_ADV];
    // diffusive_cfl = Inf selects infinite_diffusion_timescale (time_step_wizard.jl:16,80-82)
    const double dif = isinf(R[RUN_DCFL]) ? CUDART_INF : R[RUN_DCFL] * R[RUN_TAU_DIF];
    double dt = jmin(adv, dif);
    dt = jmin(R[RUN_MAX_CHANGE] * old_dt, dt);
    dt = jmax(R[RUN_MIN_CHANGE] * old_dt, dt);
    dt = jclamp(dt, R[RUN_MIN_DT], R[RUN_MAX_DT]);
    return (double)FT(dt);
}

// Grid-stride reductions for the callbacks that are due, then (last block) the clock,
// the callbacks in registration order and the loop condition.
template <typename FT>
__global__ void __launch_bounds__(256) k_sim_callbacks(SimP<FT> S, int mode, cudaGraphConditionalHandle h, int use_handle) {
    __shared__ double sh[32];
    const double* R = S.run;
    const double it_now = R[RUN_ITER] + (mode == SIM_AFTER_STEP ? 1.0 : 0.0);
    const long long itn = (long long)it_now;
    const long long wiz_every = (long long)R[RUN_WIZ_EVERY], nan_every = (long long)R[RUN_NAN_EVERY];
    const bool every = mode != SIM_AFTER_STEP;  // initialisation evaluates every callback
    const bool wiz = mode == SIM_TIMESCALES || (wiz_every > 0 && (every || itn % wiz_every == 0));
    const bool nan = mode != SIM_TIMESCALES && nan_every > 0 && (every || itn % nan_every == 0);
    const GridP<FT>& g = S.g;
    double inv = 0.0, numax = -CUDART_INF, kapmax = -CUDART_INF;
    bool bad = false;
    if (wiz || nan) {
        Met<FT> M(g);
        const size_t plane = (size_t)g.Nx * g.Ny, n = plane * g.Nz;
        for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
            const FT uu = S.u[t];
            if (wiz) {
                const int k = (int)(t / plane);
                FT a = fabs(uu) * g.rdx + fabs(S.v[t]) * g.rdy;
                if (!g.flatz) a = a + fabs(S.w[t]) * M.rdzf(k);
                inv = jmax(inv, (double)a);
                if (S.closure != GBO_CLOSURE_NONE) numax = jmax(numax, (double)S.nu[t]);
                if (S.closure == GBO_CLOSURE_AMD || S.closure == GBO_CLOSURE_SCALAR_DIFFUSIVITY)
                    for (int q = 0; q < S.ntr; ++q) kapmax = jmax(kapmax, (double)S.kap[q][t]);
            }
            if (nan) bad |= isnan(uu);
        }
    }
    inv = block_max(inv, sh);
    numax = block_max(numax, sh);
    kapmax = block_max(kapmax, sh);
    const int anybad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        double* p = S.part + (size_t)blockIdx.x * SIM_PARTS;
        p[0] = inv;
        p[1] = numax;
        p[2] = kapmax;
        p[3] = anybad ? 1.0 : 0.0;
    }
    if (!last_block(S.cnt)) return;
    // combine the partials (every thread of the last block takes a stride)
    double a0 = 0.0, a1 = -CUDART_INF, a2 = -CUDART_INF, a3 = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        const double* p = S.part + (size_t)b * SIM_PARTS;
        a0 = jmax(a0, ldcg(p));
        a1 = jmax(a1, ldcg(p + 1));
        a2 = jmax(a2, ldcg(p + 2));
        a3 = jmax(a3, ldcg(p + 3));
    }
    a0 = block_max(a0, sh);
    a1 = block_max(a1, sh);
    a2 = block_max(a2, sh);
    a3 = block_max(a3, sh);
    if (threadIdx.x != 0) return;
    double* W = S.run;
    if (wiz) {
        // the minimum of 1/x over cells is 1/(max x): rounding is monotone
        W[RUN_TAU_ADV] = (double)(FT(1) / FT(a0));
        const FT d2 = FT(W[RUN_DELTA2]);
        double dif = CUDART_INF;
        if (S.closure == GBO_CLOSURE_SMAGORINSKY_LILLY || S.closure == GBO_CLOSURE_DYNAMIC_SMAGORINSKY) {
            dif = (double)(d2 / (FT(a1) * FT(W[RUN_PR_FACTOR])));
        } else if (S.closure == GBO_CLOSURE_AMD) {
            // with no tracers the reference takes max κₑ = Inf, so Δ²/max κₑ = 0
            const FT kmax = S.ntr > 0 ? FT(a2) : FT(CUDART_INF);
            dif = jmin((double)(d2 / FT(a1)), (double)(d2 / kmax));
        } else if (S.closure == GBO_CLOSURE_SCALAR_DIFFUSIVITY) {
            // min(Δ²/ν, Δ²/max κ) with max κ = 0 without tracers
            // (turbulence_closure_diagnostics.jl:41-46)
            const FT kmax = S.ntr > 0 ? FT(a2) : FT(0);
            dif = jmin((double)(d2 / FT(a1)), (double)(d2 / kmax));
        }
        W[RUN_TAU_DIF] = dif;
    }
    if (mode == SIM_TIMESCALES) return;
    if (mode == SIM_AFTER_STEP) {
        W[RUN_TIME] = W[RUN_TIME] + W[RUN_DT];  // tick! (the clock is Float64)
        W[RUN_LAST_DT] = W[RUN_DT];
        W[RUN_ITER] = it_now;
        W[RUN_TAKEN] = W[RUN_TAKEN] + 1.0;
    }
    bool running = W[RUN_RUNNING] != 0.0;
    double reason = W[RUN_REASON];
    if (W[RUN_TIME] >= W[RUN_STOP_TIME]) {
        running = false;
        if (reason == 0.0) reason = GBO_STOP_TIME;
    }
    if (W[RUN_ITER] >= W[RUN_STOP_ITER]) {
        running = false;
        if (reason == 0.0) reason = GBO_STOP_ITERATION;
    }
    if (nan && a3 != 0.0) {
        running = false;
        W[RUN_NAN] = 1.0;
        if (reason == 0.0) reason = GBO_STOP_NAN;
    }
    if (wiz && mode != SIM_TIMESCALES && wiz_every > 0) W[RUN_SIM_DT] = wizard_dt<FT>(W, W[RUN_SIM_DT]);
    W[RUN_RUNNING] = running ? 1.0 : 0.0;
    W[RUN_REASON] = reason;
    if (use_handle) cudaGraphSetConditional(h, (running && W[RUN_TAKEN] < W[RUN_MAX_TAKEN]) ? 1u : 0u);
}
