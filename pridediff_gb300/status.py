"""Device-side timeouts, reported on the host without synchronising.

Every wait of the library's kernels on an asynchronous copy is bounded
(DD_WAIT_LIMIT polls); a wait that gives up makes its kernel skip the rest of
its work, record DD_ERR_TIMEOUT and return, so the GPU and the CUDA context
stay usable.  The record goes to two places:

* the status word in the call's workspace, read synchronously by the C ABI's
  ``dd2d_status`` / ``dd3d_status`` / ``dd2d_batch_status`` /
  ``dd_noalloc_status``;
* one word of pinned, device-mapped host memory registered with
  ``dd_set_status_sink``: the kernels write it with a system-scope atomic, so
  the host sees it by reading its own memory, with no synchronisation.

This module owns that word.  Every operator call of the package checks it
before it enqueues work (a plain host read) and raises ``RuntimeError`` if an
earlier call timed out -- the asynchronous-error model CUDA itself uses for
kernel faults.  ``device_status()`` synchronises and reports the current
state without raising.
"""
from __future__ import annotations

import threading

import torch

from . import _native as N

_lock = threading.Lock()
_word = None          # pinned int32 host tensor, shared by every device
_registered = set()   # device indices whose kernels write _word


def _sink():
    global _word
    if _word is None:
        _word = torch.zeros(1, dtype=torch.int32, pin_memory=True)
    return _word


def register(device) -> None:
    """Make the kernels on `device` write timeouts into the host word."""
    idx = torch.device(device).index
    if idx is None:
        idx = torch.cuda.current_device()
    if idx in _registered:
        return
    with _lock:
        if idx in _registered:
            return
        w = _sink()
        with torch.cuda.device(idx):
            N.check(N.load().dd_set_status_sink(w.data_ptr()), "dd_set_status_sink")
        _registered.add(idx)


def check(device) -> None:
    """Raise if a kernel timed out since the last check (no synchronisation).

    Registers the device on its first call outside a stream capture (the
    registration copies to device memory, which a capture does not allow)."""
    if not torch.cuda.is_current_stream_capturing():
        register(device)
    w = _word
    if w is None:
        return
    code = int(w[0])
    if code != N.DD_OK:
        w[0] = 0
        raise RuntimeError(f"pridediff_gb300: a kernel of an earlier call reported: {N.status_string(code)} "
                           f"(status {code}); the outputs of the calls since the last check are not valid")


def device_status(clear: bool = True) -> int:
    """Synchronise every registered device and return the recorded status
    (DD_OK or DD_ERR_TIMEOUT), clearing it if `clear`."""
    for idx in sorted(_registered):
        torch.cuda.synchronize(idx)
    if _word is None:
        return N.DD_OK
    code = int(_word[0])
    if clear:
        _word[0] = 0
    return code
