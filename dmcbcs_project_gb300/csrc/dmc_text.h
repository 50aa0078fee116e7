// Fortran formatted-output helpers shared by the walker-file and operator
// writers (host code).
#pragma once

#include <string>

namespace dmc {

// Ew.d: [-]0.<d digits>E+ee (E dropped for a three-digit exponent),
// right-justified in w columns
std::string fortran_e(double v, int w, int d);

}  // namespace dmc
