"""xara_gb300 -- GB300 implementation of the xara/OpenSees Newton-iteration hot path.

The compute path is ``libxara_gpu.so`` (hand-written sm_103a CUDA behind a C
ABI, ``include/xara_gpu.h``).  This package is the Python layer above it:

* :mod:`xara_gb300._abi`   -- ctypes mirror of the C structs;
* :mod:`xara_gb300.gpu`    -- the device model handle (element set, system,
  Newton driver, recorders, the adjoint and the direct differentiation);
* :mod:`xara_gb300.openseespy` -- the reference's OpenSeesPy modelling and
  analysis commands for the path's scope (``node``, ``fix``, ``equalDOF``,
  ``element``, ``nDMaterial``, ``uniaxialMaterial``, ``section``,
  ``pattern``, ``integrator``, ``test``, ``algorithm``, ``system``,
  ``analyze``, ``nodeDisp``) building and running a device model;
* :mod:`xara_gb300.adjoint` -- gradients of a frame response with respect
  to material parameters as a ``torch.autograd.Function`` (reverse mode by
  the adjoint, forward mode by the direct differentiation);
* :mod:`xara_gb300.tcl`    -- a Tcl subset running the reference's scripts
  for the path's scope through :mod:`xara_gb300.openseespy`;
* :mod:`xara_gb300.configs` -- seeded synthetic workloads.

There is no CPU fallback: loading the package on a machine without the
built library raises ``ImportError`` from :func:`xara_gb300.gpu.lib`.
"""
from ._abi import ModelDesc, PhaseDesc  # noqa: F401

__all__ = ["ModelDesc", "PhaseDesc"]
