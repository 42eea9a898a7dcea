// Host assembly of the Laplacian on a general (non-orthogonal) mesh with a
// tensor conductivity: OpenFOAM's "Gauss linear corrected" scheme
// (gaussLaplacianScheme::fvmLaplacian for a tensor Gamma, finiteVolume of
// OpenFOAM v2312) split into the implicit face coefficients and the
// geometric factors of the explicit correction the step kernels evaluate
// every PIMPLE corrector.
#pragma once

#include <vector>

#include "../../include/cardiac_gpu.h"

namespace cfg {

struct CorrectedOperator {
    std::vector<double> coeff;   // [nf] upper(): deltaCoeffs * SfGammaSn
    std::vector<double> w;       // [nf] linear interpolation weight of the owner
    std::vector<double> k;       // [nf][3] SfGammaCorr (+ SfGammaSn * corrVec when corrected)
    std::vector<double> g_own;   // [nf][3] weight of (phi_N - phi_P) in the owner's gradient
    std::vector<double> g_nei;   // [nf][3] weight of (phi_P - phi_N) in the neighbour's gradient
    std::vector<double> bk;      // [n][3] wall factor: sum over the cell's wall faces of
                                 // SfGammaCorr - (SfGammaCorr.n) n
};

// Fills `op` from the mesh geometry; sigma_cells ([n][6], may be null)
// overrides the uniform sigma.  Returns CFG_OK or a CFG_ERR_* code (with
// the message recorded).
int assemble_corrected(const cfg_mesh_desc* m, const double* sigma_uniform,
                       const double* sigma_cells, int grad_scheme, int uncorrected,
                       CorrectedOperator& op);

}  // namespace cfg
