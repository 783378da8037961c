"""Branch stamps on the device (p3s/models/TwoPort.py, TransmissionLineModel.py,
TwoWindingTransformerModel.py): the general two-port with complex ratios at both ends,
out-of-service masking and Kron elimination of open ends, computed per branch by the
``gbpf_branch_stamps`` kernel; ``GpuSolver.update_Y_from_branches`` sums them into the
resident Ybus. The element tables' unit conversions (ohm/km, nF/km, rated voltages) stay with
the caller, as in the reference's model constructors."""

from __future__ import annotations

import numpy as np

from . import _lib


def _c(a, m):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.complex128), (m,)))


def _u(a, m):
    return None if a is None else np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.uint8), (m,)))


def branch_stamps(ys, y_from=0.0, y_to=0.0, a=1.0, b=1.0, in_service=None, open_from=None, open_to=None):
    """(m, 4) complex stamps (Yff, Yft, Ytf, Ytt): ys series admittance (p.u.), y_from / y_to
    shunt admittance at each end, a / b complex ratios at each end (tap * exp(j shift))."""
    ys = np.ascontiguousarray(np.asarray(ys, dtype=np.complex128).ravel())
    m = len(ys)
    arrs = [_c(x, m) for x in (ys, y_from, y_to, a, b)]
    flags = [_u(x, m) for x in (in_service, open_from, open_to)]
    out = np.empty((m, 4), dtype=np.complex128)
    rc = _lib.require_device().gbpf_branch_stamps(m, *[_lib.cview(x) for x in arrs],
                                                  *[None if f is None else _lib.u8(f) for f in flags], _lib.cview(out))
    _lib.check(rc, "branch_stamps")
    return out
