"""psc — host-side Python bindings of the GB300 strong-connectivity library.

The compute path is libpsc_cuda.so (hand-written sm_103a kernels behind the C
ABI in include/psc.h); this package only loads it, builds inputs with
libpsc_host.so and exposes the calls.  There is no CPU fallback.
"""
from ._lib import Params, PscError, Stats, cuda, host, strerror  # noqa: F401
from .graph import (DeviceGraph, HostGraph, batch_member, batch_member_spec,  # noqa: F401
                    batch_workload, default_params, random_permutation)
from .server import Server, server_config  # noqa: F401
