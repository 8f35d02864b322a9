"""Device context: one kr_ctx per process and GPU, torch for buffers and streams."""
import ctypes
import threading

import torch

from . import _native

_ctx = {}
_lock = threading.Lock()


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("richmol_gb300 needs a CUDA GPU (GB300, sm_103a); no CPU fallback exists")


def context(device=None):
    """The kr_ctx handle of ``device`` (default: torch's current device)."""
    require_cuda()
    dev = torch.cuda.current_device() if device is None else int(device)
    with _lock:
        if dev not in _ctx:
            h = ctypes.c_void_p()
            _native.check(_native.lib().kr_ctx_create(dev, ctypes.byref(h)))
            _ctx[dev] = h
        return _ctx[dev]


def stream_ptr(stream=None):
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)
