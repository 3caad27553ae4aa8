"""Field post-processing on the GPU, mirroring sucemfem.PostProcessing: the
field at points (``Reconstruct``), the EM functional
(``CalcEMFunctional``), the power flux through the boundary
(``power_flux.SurfaceFlux``, ``power_flux.VariationalSurfaceFlux``) and the
near-to-far-field transforms (``surface_ntff.NTFF``,
``variational_ntff.NTFF``)."""
from .PostProcessing import CalcEMFunctional, Reconstruct  # noqa: F401
