"""Field post-processing on the GPU: the field at points
(``PostProcessing.Reconstruct``) and the power flux through the boundary
(``power_flux.SurfaceFlux``), mirroring sucemfem.PostProcessing."""
from .PostProcessing import Reconstruct  # noqa: F401
