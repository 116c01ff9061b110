// eigen.h -- lowest eigenmodes at the current state (see eigen.cpp).
#pragma once

#include <vector>

#include "engine.h"
#include "host_model.h"

namespace fgpu {

// The nmod lowest eigenvalues lambda of K phi = lambda M phi of model 0 of the
// engine at its current configuration (ascending) and their M-orthonormal
// eigenvectors (equation order, nmod columns of neq).  nNeg: eigenvalues below
// zero.  Returns 0, 1 when not every mode reached the tolerance (results still
// given), < 0 on error (-3: singular stiffness matrix).  Only between steps.
int lowestModes(Engine& eng, const HostModel& m, int nmod, std::vector<double>& lambda, std::vector<double>& vecs,
                int& nNeg);

// the mass matrix over the free equations in the model's CSR pattern, element
// mass matrices rotated with the given frames (12 per element)
void massCsr(const HostModel& m, const std::vector<double>& frames, std::vector<double>& vals);

}  // namespace fgpu
