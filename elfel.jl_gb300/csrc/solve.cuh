// Device solvers for K[1:nu,1:nu] x = F[1:nu] - (K*T)[1:nu].
#pragma once
#include "sysmat.cuh"

namespace elfel {

void solver_release(Ctx* c, elfel_sysmat* m);

}  // namespace elfel
