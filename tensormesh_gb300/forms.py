"""Recognition of integrands on the GPU path.

The reference accepts any ``forward`` and evaluates it through nested
``vmap`` (assemble/element_assembler.py:328-398).  The GPU path compiles no
user code: it implements the built-in integrands as CUDA kernels and maps a
user ``forward`` onto one of them by *probing* it -- the forward is called on
small random arguments shaped exactly as ``vmap`` would pass them (``u, v``
scalars, ``gradu, gradv`` [D] vectors, a coefficient scalar) and its output
is matched against each candidate integrand; the match must hold to rounding
on several independent probes.  Anything else raises NotImplementedError
(there is no CPU fallback).

Bilinear candidates:  c * (gradu . gradv)      (builtin.py:62-63)
                      c * u * v                (builtin.py:100-101)
                      c * Ba^T C(nu) Bb        (builtin.py:173-179)
Linear candidates:    c * v, c in R^H          (builtin.py:886-927)
                      f(x) * v                 (builtin.py:929-969)
                      f * v, f point data      (node_assembler.py:389)
"""
from __future__ import annotations

import inspect
from dataclasses import dataclass
from typing import Optional

import torch

_TOL = 1e-11


@dataclass
class BilinearForm:
    kind: str                     # "laplace" | "mass" | "elasticity"
    coef_key: Optional[str]       # argument name carrying the coefficient, if any
    scale: float = 1.0            # constant factor of the integrand
    lam: float = 0.0              # elasticity: Lame lambda per unit coefficient
    mu: float = 0.0               # elasticity: Lame mu per unit coefficient


def reference_lame(E: float, nu: float):
    """Lame constants exactly as the reference forms them: computed in Python
    floats, then wrapped by ``torch.tensor`` (functional/elasticity.py:
    259-266), i.e. rounded to torch's default dtype (float32 unless the
    caller changed it) before being cast to the assembly dtype."""
    mu = E / (2.0 * (1.0 + nu))
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return float(torch.tensor(lam)), float(torch.tensor(mu))


@dataclass
class LinearForm:
    kind: str                     # "const" | "func" | "point"
    coef_key: Optional[str] = None
    const: Optional[torch.Tensor] = None  # [H] for "const"
    func: Optional[object] = None         # callable of x for "func"
    n_comp: int = 1


def _close(a: torch.Tensor, b: torch.Tensor) -> bool:
    a = torch.as_tensor(a, dtype=torch.float64)
    b = torch.as_tensor(b, dtype=torch.float64)
    if a.shape != b.shape:
        return False
    scale = max(1.0, float(b.abs().max()) if b.numel() else 1.0)
    return bool(((a - b).abs() <= _TOL * scale).all())


def elasticity_block(g: torch.Tensor, h: torch.Tensor, lam: float, mu: float) -> torch.Tensor:
    """Ba^T C Bb for gradients g, h [D]: lam g_a h_b + mu (delta_ab g.h + g_b h_a)."""
    D = g.shape[0]
    return lam * torch.outer(g, h) + mu * (torch.eye(D, dtype=g.dtype) * (g @ h) + torch.outer(h, g))


def recognise_bilinear(fn, dim: int, coef_keys) -> BilinearForm:
    params = list(inspect.signature(fn).parameters)
    allowed = {"u", "v", "gradu", "gradv"}
    extra = [p for p in params if p not in allowed]
    if len(extra) > 1 or (extra and extra[0] not in coef_keys):
        raise NotImplementedError(
            f"forward{tuple(params)}: the GPU path supports at most one coefficient argument drawn from "
            f"element_data/point_data/scalar_data")
    ckey = extra[0] if extra else None
    gen = torch.Generator().manual_seed(1234)
    probes = []
    for _ in range(4):
        args = {"u": torch.rand((), generator=gen, dtype=torch.float64) + 0.5,
                "v": torch.rand((), generator=gen, dtype=torch.float64) + 0.5,
                "gradu": torch.randn(dim, generator=gen, dtype=torch.float64),
                "gradv": torch.randn(dim, generator=gen, dtype=torch.float64)}
        c = torch.rand((), generator=gen, dtype=torch.float64) + 0.5
        if ckey:
            args[ckey] = c
        with torch.no_grad():
            out = fn(*[args[p] for p in params])
        probes.append((args, (c if ckey else torch.tensor(1.0, dtype=torch.float64)), torch.as_tensor(out)))
    out0 = probes[0][2]
    if out0.dim() == 0:
        for kind, f in (("laplace", lambda a: a["gradu"] @ a["gradv"]), ("mass", lambda a: a["u"] * a["v"])):
            ratios = [float(o / (c * f(a))) for a, c, o in probes if abs(float(c * f(a))) > 1e-3]
            if ratios and all(abs(r - ratios[0]) <= _TOL * max(1, abs(ratios[0])) for r in ratios):
                if all(_close(o, ratios[0] * c * f(a)) for a, c, o in probes):
                    return BilinearForm(kind, ckey, ratios[0])
    elif out0.shape == (dim, dim):
        a, c, o = probes[0]
        g, h = a["gradu"], a["gradv"]
        # least squares for (lam', mu') in o = lam' A + mu' Bm
        A = torch.outer(g, h).reshape(-1)
        Bm = (torch.eye(dim, dtype=g.dtype) * (g @ h) + torch.outer(h, g)).reshape(-1)
        M = torch.stack([A, Bm], 1)
        sol = torch.linalg.lstsq(M, (o / c).reshape(-1, 1)).solution.reshape(-1)
        lam, mu = float(sol[0]), float(sol[1])
        if mu != 0.0 and all(_close(o2, c2 * elasticity_block(a2["gradu"], a2["gradv"], lam, mu))
                             for a2, c2, o2 in probes):
            return BilinearForm("elasticity", ckey, 1.0, lam, mu)
    raise NotImplementedError(
        f"forward{tuple(params)} is not one of the integrands built for the GPU path "
        f"(c*gradu@gradv, c*u*v, c*Ba^T C Bb)")


def recognise_linear(fn, dim: int, point_keys, scalar_keys) -> LinearForm:
    params = list(inspect.signature(fn).parameters)
    if "v" not in params:
        raise NotImplementedError(f"forward{tuple(params)}: a linear form must take v")
    others = [p for p in params if p != "v"]
    gen = torch.Generator().manual_seed(4321)
    v1 = torch.tensor(1.0, dtype=torch.float64)
    v2 = torch.tensor(2.5, dtype=torch.float64)
    if not others:
        with torch.no_grad():
            o1 = torch.as_tensor(fn(v1), dtype=torch.float64)
            o2 = torch.as_tensor(fn(v2), dtype=torch.float64)
        if _close(o2, 2.5 * o1) and o1.dim() <= 1:
            c = o1.reshape(-1)
            return LinearForm("const", const=c, n_comp=int(c.numel()))
    elif others == ["x"] or (len(others) == 1 and others[0] == "x"):
        x = torch.rand(dim, generator=gen, dtype=torch.float64)
        with torch.no_grad():
            o1 = torch.as_tensor(fn(x, v1) if params.index("x") < params.index("v") else fn(v1, x))
            o2 = torch.as_tensor(fn(x, v2) if params.index("x") < params.index("v") else fn(v2, x))
        if _close(o2, 2.5 * o1):
            xi = params.index("x")
            vi = params.index("v")

            def g(xx, _fn=fn, _xi=xi, _vi=vi):
                args = [None, None]
                args[_xi] = xx
                args[_vi] = torch.ones((), dtype=xx.dtype, device=xx.device)
                return _fn(*args)
            return LinearForm("func", func=g, n_comp=int(o1.numel()))
    elif len(others) == 1 and (others[0] in point_keys or others[0] in scalar_keys):
        key = others[0]
        f = torch.rand((), generator=gen, dtype=torch.float64) + 0.5
        order = params

        def call(vv, ff):
            return fn(*[vv if p == "v" else ff for p in order])
        with torch.no_grad():
            o1 = torch.as_tensor(call(v1, f))
            o2 = torch.as_tensor(call(v2, 2.0 * f))
        if _close(o2, 5.0 * o1) and _close(o1, f * torch.ones_like(o1) * (o1 / f)):
            ratio = float(o1.reshape(-1)[0] / f)
            kind = "point" if key in point_keys else "scalar"
            return LinearForm(kind, coef_key=key, const=torch.tensor([ratio], dtype=torch.float64), n_comp=1)
    raise NotImplementedError(f"forward{tuple(params)} is not one of the load integrands built for the GPU path")
