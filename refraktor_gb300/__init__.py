"""GB300-native fractal-flame hot path (chaos game, tonemap, density blur,
Catmull-Rom genome interpolation) behind librefrakt's plugin surface.

`refraktor_gb300.librefrakt` mirrors the reference's C++ interface over the C
ABI of librfk.so (include/rfk.h); `refraktor_gb300.build` compiles it.
"""
from . import build  # noqa: F401

__all__ = ["build", "librefrakt", "synthetic"]
