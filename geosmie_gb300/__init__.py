"""GB300-native (sm_103a) Mie hot path of GEOSmie.

Drop-ins for the reference's Python API:
  geosmie_gb300.Mie, geosmie_gb300.MultipleMie   pymiecoated.Mie / MultipleMie
  geosmie_gb300.table                            runoptics / dointegration.fun
  geosmie_gb300.gsf                              rungsf / convertncdf (pygeos)
All arithmetic runs in libgbmie.so (include/gbmie.h); there is no CPU path.
"""
from .mie import Mie, MultipleMie, Cache  # noqa: F401

__all__ = ["Mie", "MultipleMie", "Cache"]
