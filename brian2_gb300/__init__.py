"""GB300-native clock-driven step loop for Brian2 (``set_device('b200')``).

* :mod:`brian2_gb300.runtime` -- ctypes host of the C ABI (include/b200.h);
* :mod:`brian2_gb300.codegen` -- network spec -> fused persistent CUDA kernel;
* :mod:`brian2_gb300.construct` -- Brian-identical host construction;
* :mod:`brian2_gb300.scale` -- device-side construction of very large networks;
* :mod:`brian2_gb300.batched` -- parameter sweeps in one persistent launch;
* :mod:`brian2_gb300.adjoint` -- exact-linear LIF adjoint (torch.autograd);
* :mod:`brian2_gb300.brian_device` -- the Brian2 device plugin (needs brian2).
"""
import sys

__version__ = "0.1.0"


def register_brian_device():
    """Registers ``b200`` in Brian2's device table (imports brian2)."""
    from . import brian_device  # noqa: F401
    return brian_device.b200_device


if "brian2" in sys.modules:
    try:
        register_brian_device()
    except ImportError:
        pass
