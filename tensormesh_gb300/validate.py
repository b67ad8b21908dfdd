"""Host-side input validation with clear errors.

The reference indexes its tensors with the connectivity directly and fails
deep inside torch (or silently reads another row) when an element lists a
node that does not exist; non-finite coefficients flow through to NaN
matrices.  Here both are rejected before any kernel launch:

* connectivity: every index in [0, n_points), checked once per mesh when the
  pattern is built (``IndexError``);
* floating inputs of a call (points, per-element / per-point / per-quadrature
  coefficients): all finite (``ValueError`` naming the input).  This check
  reads the inputs on the device and waits for the answer (one host
  synchronisation per call); ``set_input_checks(False)`` turns it off for
  callers that pipeline many calls and validate their data elsewhere.
"""
from __future__ import annotations

from typing import Iterable, Optional, Tuple

import torch

_CHECK_FINITE = True


def set_input_checks(enabled: bool) -> None:
    """Turn the per-call finiteness check on or off (on by default)."""
    global _CHECK_FINITE
    _CHECK_FINITE = bool(enabled)


def input_checks_enabled() -> bool:
    return _CHECK_FINITE


def check_connectivity(elements: torch.Tensor, n_points: int) -> None:
    if elements.numel() == 0:
        return
    lo, hi = int(elements.min()), int(elements.max())
    if lo < 0 or hi >= n_points:
        bad = lo if lo < 0 else hi
        row = int(torch.nonzero((elements < 0) | (elements >= n_points), as_tuple=True)[0][0])
        raise IndexError(f"element {row} refers to node {bad}, outside [0, {n_points}) "
                         f"(the mesh has {n_points} points)")


def check_finite(items: Iterable[Tuple[str, Optional[torch.Tensor]]]) -> None:
    if not _CHECK_FINITE:
        return
    named = [(n, t) for n, t in items if t is not None and torch.is_tensor(t) and t.is_floating_point() and t.numel()]
    if not named:
        return
    flags = torch.stack([torch.isfinite(t.detach()).all() for _, t in named])
    if bool(flags.all()):
        return
    first = int(torch.nonzero(~flags, as_tuple=True)[0][0])
    raise ValueError(f"{named[first][0]} holds a non-finite value (nan or inf)")
