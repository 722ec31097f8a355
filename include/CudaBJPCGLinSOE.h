// CudaBJPCGLinSOE: `system CudaBJPCG <rtol> <maxit>`, the reference's
// LinearSOE with SparseGenColLinSOE's assembly
// (system_of_eqn/linearSOE/sparseGEN/SparseGenColLinSOE.cpp:161-350) and a
// block-Jacobi preconditioned CG on the device (xg_linsoe_*, XG_SYSTEM_BJPCG).
// The body is CudaLinSOE (CudaLinSOE.h).
#ifndef XARA_CUDA_BJPCG_LINSOE_H
#define XARA_CUDA_BJPCG_LINSOE_H

#include "CudaLinSOE.h"

class CudaBJPCGLinSOE : public CudaLinSOE {
 public:
  explicit CudaBJPCGLinSOE(double rtol = 1e-12, int maxit = 20000, int classTag = 0)
      : CudaLinSOE(XG_SYSTEM_BJPCG, rtol, maxit, classTag) {}
};

#endif  // XARA_CUDA_BJPCG_LINSOE_H
