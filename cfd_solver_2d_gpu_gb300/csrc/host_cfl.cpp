// The driver's adaptive CFL (input.toml time.strategy = 1): host logic of
// RoutineController (FVMR/src/drivers/RoutineController.h:5-83, RoutineController.cpp:
// 13-90), applied by CDriver::start at each print event with the residual of rho
// (FVMR/src/drivers/CDriver.cpp:115-120).
//
//   - the first call records the residual;
//   - after step 1000, a residual above 10x the record scales CFL by 0.75 (at most once
//     every 500 steps);
//   - after step 5000, a residual below half the record scales CFL by 1.1 and the record
//     by 0.9, and in any case CFL is scaled by 1.05; both share one 1000-step cool-down;
//   - CFL is kept at or above 0.5.
#include "internal.h"

struct fvgb_cfl_controller {
    struct Action {  // a change that may be made again only after its cool-down
        int cold = 1000, last = 0;
        bool try_scale(double& v, int now, double factor) {
            if (now - last < cold) return false;
            v *= factor;
            last = now;
            return true;
        }
    };
    int strategy = 0;
    int calls = 0;
    double record = 10.0;
    Action increase{1000, 0}, decrease{500, 0};
};

using namespace fvgb;

extern "C" int fvgb_cfl_controller_create(int strategy, fvgb_cfl_controller** out) {
    if (!out) return fail(FVGB_ERR_ARG, "null argument");
    if (strategy != 0 && strategy != 1) return fail(FVGB_ERR_ARG, "time.strategy is 0 (none) or 1 (adaptive CFL)");
    *out = new fvgb_cfl_controller();
    (*out)->strategy = strategy;
    return 0;
}

extern "C" int fvgb_cfl_controller_apply(fvgb_cfl_controller* c, double residual_rho, int step, double* CFL,
                                         int* applied) {
    if (!c || !CFL) return fail(FVGB_ERR_ARG, "null argument");
    bool ok = false;
    if (c->strategy == 1) {
        if (c->calls == 0) {
            c->record = residual_rho;
        } else {
            if (step > 1000 && residual_rho > c->record * 10.0 && c->decrease.try_scale(*CFL, step, 0.75)) ok = true;
            if (step > 5000 && residual_rho < c->record * 0.5 && c->increase.try_scale(*CFL, step, 1.1)) {
                c->record *= 0.9;
                ok = true;
            }
            if (step > 5000 && c->increase.try_scale(*CFL, step, 1.05)) ok = true;
            if (*CFL < 0.5) *CFL = 0.5;
        }
        c->calls++;
    }
    if (applied) *applied = ok ? 1 : 0;
    return 0;
}

extern "C" void fvgb_cfl_controller_destroy(fvgb_cfl_controller* c) { delete c; }
