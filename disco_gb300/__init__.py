"""GB300-native (sm_103a) implementation of Disco's moving-mesh RK substep
cycle behind a C ABI (include/disco_gpu.h).  See `disco_gb300.api`."""
from .api import (Batch, Domain, HostDomain, DiscoError, Mlp, read_params, read_modules,  # noqa: F401
                  lib)

__all__ = ["Batch", "Domain", "HostDomain", "DiscoError", "Mlp", "read_params", "read_modules", "lib"]
