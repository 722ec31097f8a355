// CudaProfileSPDLinSOE: `system ProfileSPD` with the factorisation on the
// device.  Replaces ProfileSPDLinSOE + ProfileSPDLinDirectSolver
// (system_of_eqn/linearSOE/profileSPD/ProfileSPDLinSOE.cpp:115-410,
// ProfileSPDLinDirectSolver.cpp:100-420; the reference's default system,
// runtime/runtime/BasicAnalysisBuilder.cpp:820):
//
//   * addA keeps the terms with row <= col in ProfileSPDLinSOE::addA's
//     order (column-outer, row-inner), so the values the factorisation reads
//     equal the reference's profile bit for bit;
//   * solve factors once per matrix (the reference's isAfactored: again only
//     after zeroA or addA) with the device LDL' and the reference's pivot
//     checks (a first pivot <= 0, a pivot == 0 or |pivot| <= 1e-12 fail the
//     solve), then runs the substitutions; DisplacementControl's second
//     right-hand side per iteration reuses the factors.
//
// The body is CudaLinSOE (CudaLinSOE.h); xg_linsoe_* with XG_SYSTEM_PROFILE_SPD.
#ifndef XARA_CUDA_PROFILESPD_LINSOE_H
#define XARA_CUDA_PROFILESPD_LINSOE_H

#include "CudaLinSOE.h"

class CudaProfileSPDLinSOE : public CudaLinSOE {
 public:
  explicit CudaProfileSPDLinSOE(int classTag = 0)
      : CudaLinSOE(XG_SYSTEM_PROFILE_SPD, 1e-12, 1, classTag) {}
};

#endif  // XARA_CUDA_PROFILESPD_LINSOE_H
