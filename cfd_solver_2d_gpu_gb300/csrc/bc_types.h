// Boundary type codes (FVMR/src/global/Constexpr.h:39-57), shared by host and device code.
#pragma once

namespace fvgb {

enum BcType : int {
    BC_INTERIOR = -1,
    BC_WALL_NONVISCOUS = 6001,  // slip wall
    BC_WALL_ADIABAT = 6002,     // no-slip adiabatic wall
    BC_WALL_ISOTHERMAL = 6003,  // no-slip isothermal wall (named by the reference, given no flux)
    BC_INLET = 6011,
    BC_OUTLET = 6012,
    BC_INF = 6013,              // far field
    BC_DSR = 6014,              // double Mach reflection
    BC_SYMMETRY = 6021,
    BC_PERIODIC_0 = 6100,
    BC_PERIODIC_9 = 6109,
};

}  // namespace fvgb
