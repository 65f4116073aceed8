"""GB300-native batched SSP/CSP path of OpenSPS behind its C API.

``libopensps_gb300/_lib/libopensps_gb300.so`` is the product: the ``opensps.h`` entry points of the batched CSP
path over hand-written sm_103a kernels. This package builds it (:mod:`.build`), binds it through ctypes
(:mod:`.capi`), writes the synthetic libraries of the benchmark workloads (:mod:`.synthdata`) and wraps the gradient
path as a ``torch.autograd.Function`` (:mod:`.torch_ops`).
"""
from .capi import Context, OpenSPSError, load_library, library_path  # noqa: F401

__all__ = ["Context", "OpenSPSError", "load_library", "library_path"]
