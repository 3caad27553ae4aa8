from .Interpolation import SurfaceInterpolant  # noqa: F401
