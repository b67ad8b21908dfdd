"""ElementAssembler / NodeAssembler with the reference's interface, backed by
the CUDA patch-assembly kernels.

Interface parity (TensorMesh):
  * ``ElementAssembler.from_mesh(mesh, quadrature_order=2, project='reduce',
    *args, **kwargs)`` (assemble/element_assembler.py:789-909),
    ``from_assembler`` (:759-787), ``__post_init__`` hook, and
    ``__call__(points=None, func=None, point_data=None, element_data=None,
    scalar_data=None, batch_size=-1) -> SparseMatrix`` (:243-466);
  * ``NodeAssembler.from_mesh`` / ``from_elements`` / ``from_assembler`` and
    ``__call__(points=None, func=None, point_data=None, scalar_data=None,
    batch_size=1) -> Tensor[N*H]`` (assemble/node_assembler.py:242-738);
  * the built-ins ``LaplaceElementAssembler``, ``MassElementAssembler``,
    ``LinearElasticityElementAssembler(E, nu)``, ``const_node_assembler``,
    ``func_node_assembler`` (assemble/builtin.py).

Error behaviour follows the reference: AssertionError for shape mismatches,
ValueError for a forward parameter that no data provides
(element_assembler.py:364), NotImplementedError for an integrand that has no
GPU kernel.  ``batch_size`` is accepted and ignored: it is a memory knob of
the reference's quadrature chunking, and the fused kernel never materialises
per-quadrature-point tensors.
"""
from __future__ import annotations

import inspect
import threading
from typing import Callable, Dict, Mapping, Optional

import torch
import torch.nn as nn

from . import _lib, element as E_, forms as F_
from .plan import PatchPlan, block_pattern, node_pattern
from .sparse import SparseMatrix
from .validate import check_connectivity

PRECISION = {"emulated": _lib.TM_PREC_EMULATED, "native": _lib.TM_PREC_NATIVE}


class MeshTopology:
    """Pattern + patch plan of one connectivity, shared by every assembler
    built on it (the analogue of the reference's ``edges`` + projector)."""

    def __init__(self, elements: torch.Tensor, points: torch.Tensor, element_type: str):
        self.element_type = element_type
        self.el_id, self.dim, self.n_basis, _ = E_.element_info(element_type)
        assert elements.dim() == 2, f"the connectivity should be [n_element, n_basis], but got {tuple(elements.shape)}"
        assert elements.shape[1] == self.n_basis, \
            f"{element_type} elements have {self.n_basis} nodes, but the connectivity has {elements.shape[1]} columns"
        check_connectivity(elements, int(points.shape[0]))
        self.elements = elements.to(torch.int32).contiguous()
        self._elements_long = elements.long()
        self.n_points = int(points.shape[0])
        self.n_elements = int(elements.shape[0])
        self.timings = {}  # seconds of the pattern build and of each patch plan (device work included)
        t0 = _now(elements.device)
        self.pattern = node_pattern(elements, self.n_points)
        self.timings["pattern_s"] = _now(elements.device) - t0
        self._coords = points.detach()
        self._plans = {}
        self.plan, self._plan_struct = self.plan_for(1)
        self._block = {}
        self._incidence = None

    # accumulator budget per patch in node slots (the scalar forms' kernels
    # autotune it; 3x3 blocks: 512 slots = 36 KB of accumulators, so three
    # elasticity CTAs fit an SM)
    _SLOT_BUDGET = {1: 6144, 2: 1600, 3: 512}

    def plan_for(self, H: int, budget: int = None):
        """(PatchPlan, ctypes struct) sized for H x H block slots (or for an
        explicit accumulator budget in node slots)."""
        if budget is None:
            budget = self._SLOT_BUDGET.get(H, max(64, 6144 // (H * H)))
        if budget not in self._plans:
            t0 = _now(self._coords.device)
            plan = PatchPlan(self._elements_long, self._coords, self.pattern, slot_budget=budget)
            self._plans[budget] = (plan, plan.to_struct())
            self.timings[f"plan_{budget}_s"] = _now(self._coords.device) - t0
        return self._plans[budget]

    def dof_pattern(self, H: int):
        if H not in self._block:
            self._block[H] = block_pattern(self.pattern.indptr, self.pattern.indices, H)
        return self._block[H]

    @property
    def plan_struct(self):
        return self._plan_struct


def _now(device) -> float:
    """Host time after the device has finished its queued work."""
    import time
    if torch.device(device).type == "cuda":
        torch.cuda.synchronize(device)
    return time.perf_counter()


_TOPO_CACHE: Dict[tuple, MeshTopology] = {}
_TOPO_LOCK = threading.Lock()


def topology_for(elements: torch.Tensor, points: torch.Tensor, element_type: str) -> MeshTopology:
    key = (elements.data_ptr(), tuple(elements.shape), str(elements.device), elements._version,
           int(points.shape[0]), element_type)
    with _TOPO_LOCK:
        topo = _TOPO_CACHE.get(key)
        if topo is None:
            topo = MeshTopology(elements, points, element_type)
            if len(_TOPO_CACHE) > 8:
                _TOPO_CACHE.pop(next(iter(_TOPO_CACHE)))
            _TOPO_CACHE[key] = topo
        return topo


def _require_cuda(t: torch.Tensor, what: str):
    if not t.is_cuda:
        raise RuntimeError(f"tensormesh_gb300 runs on CUDA devices only ({what} is on {t.device}); "
                           "there is no CPU fallback")


def _dtype_code(dtype: torch.dtype) -> int:
    if dtype == torch.float64:
        return _lib.TM_F64
    if dtype == torch.float32:
        return _lib.TM_F32
    raise TypeError(f"unsupported dtype {dtype} (float32 or float64)")


def _mesh_single_type(mesh):
    elements = mesh.elements()
    if isinstance(elements, dict):
        if len(elements) != 1:
            raise NotImplementedError("mixed element types are not on the GPU path")
        (etype, elements), = elements.items()
    else:
        etype = mesh.default_element_type
    return etype, elements


def launch_assemble(topo: MeshTopology, form_code: int, points: torch.Tensor, out: torch.Tensor, *,
                    quadrature_order: int, coef_kind: int = _lib.TM_COEF_SCALAR, coef=None,
                    scal=(1.0, 0.0, 0.0), lame=(0.0, 0.0), n_comp: int = 1, precision: str = "emulated",
                    slot_budget: int = None):
    tables = E_.kernel_tables(topo.element_type, quadrature_order, points.device)
    a = _lib.AssembleArgs()
    a.element = topo.el_id
    a.form = form_code
    a.dtype = _dtype_code(points.dtype)
    a.precision = PRECISION[precision]
    a.coef_kind = coef_kind
    a.n_comp = n_comp
    a.n_quad = E_.n_quadrature(topo.element_type, quadrature_order)
    a.tables = tables.data_ptr()
    a.points = points.data_ptr()
    a.coef = 0 if coef is None else coef.data_ptr()
    for i in range(3):
        a.scal[i] = float(scal[i]) if i < len(scal) else 0.0
    a.lam, a.mu = float(lame[0]), float(lame[1])
    a.out = out.data_ptr()
    H = n_comp if form_code == _lib.TM_FORM_LOAD else (topo.dim if form_code == _lib.TM_FORM_ELASTICITY else 1)
    plan = topo.plan_for(1 if form_code == _lib.TM_FORM_LOAD else H, slot_budget)[1]
    _lib.call("tm_assemble", plan, a, _lib.stream_handle(points.device))
    return tables  # keep alive until the stream consumes it


class _AssemblerDevice:
    """``device`` / ``dtype`` / ``type(dtype)`` of the reference assemblers
    (element_assembler.py:172-194, node_assembler.py): the stored points
    carry both; ``type`` casts them (float32 or float64)."""

    @property
    def device(self) -> torch.device:
        return self.points.device

    @property
    def dtype(self) -> torch.dtype:
        return self.points.dtype

    def type(self, dtype: torch.dtype):
        if dtype not in (torch.float32, torch.float64):
            raise TypeError(f"the dtype {dtype} is not supported (float32 or float64)")
        self.points = self.points.to(dtype)
        return self


class ElementAssembler(_AssemblerDevice, nn.Module):
    """Assemble a bilinear form into a global CSR matrix on the GPU."""

    _builtin_form: Optional[F_.BilinearForm] = None
    precision = "emulated"   # FP64 arithmetic: "emulated" (double-float) or "native"
    slot_budget = None       # patch accumulator budget (node slots); None = default, see autotune()

    def __init__(self, topology: MeshTopology, points: torch.Tensor, quadrature_order: int, *args, **kwargs):
        super().__init__()
        self.topology = topology
        self.quadrature_order = int(quadrature_order)
        self.register_buffer("points", points, persistent=False)
        self.element_types = [topology.element_type]
        self.n_points = topology.n_points
        self._form_cache = {}
        self.__post_init__(*args, **kwargs)

    def __post_init__(self, *args, **kwargs):
        pass

    @classmethod
    def from_mesh(cls, mesh, quadrature_order: int = 2, project: str = "reduce", *args, **kwargs):
        assert project in ("reduce", "sparse")
        etype, elements = _mesh_single_type(mesh)
        points = mesh.points
        topo = topology_for(elements.to(points.device), points, etype)
        return cls(topo, points, quadrature_order, *args, **kwargs)

    @classmethod
    def from_assembler(cls, obj: "ElementAssembler", *args, **kwargs):
        assert isinstance(obj, ElementAssembler), f"obj must be an instance of ElementAssembler, but got {type(obj)}"
        return cls(obj.topology, obj.points, obj.quadrature_order, *args, **kwargs)

    def energy(self, points: Optional[torch.Tensor] = None, func=None, point_data=None, element_data=None,
               scalar_data=None, batch_size: int = -1):
        """Total energy sum_e sum_q psi w |det J| (element_assembler.py:468-680).

        Runs on the GPU kernels for the Neo-Hookean density of
        ``NeoHookeanModel`` with ``point_data={"displacement": u}``; the result
        is differentiable with respect to u (``.backward()`` leaves the
        internal force vector in ``u.grad``).  Other densities raise
        ``NotImplementedError`` (there is no CPU fallback).  ``batch_size`` is
        accepted and ignored, as for ``__call__``."""
        from .energy import NeoHookeanModel, neo_hookean_energy
        density = func if func is not None else getattr(self, "element_energy", None)
        is_nh = (isinstance(self, NeoHookeanModel) and
                 getattr(density, "__func__", None) is NeoHookeanModel.element_energy)
        if not is_nh:
            raise NotImplementedError("energy assembly on the GPU supports the Neo-Hookean density "
                                      "(NeoHookeanModel.element_energy)")
        point_data = dict(point_data or {})
        point_data.pop("x", None)
        if set(point_data) != {"displacement"} or element_data or scalar_data:
            raise NotImplementedError("the Neo-Hookean energy takes point_data={'displacement': u} only")
        return neo_hookean_energy(self, point_data["displacement"], points, self.mu, self.lam)

    @property
    def elements(self):
        return {self.topology.element_type: self.topology.elements}

    @property
    def edges(self) -> torch.Tensor:
        p = self.topology.pattern
        rows = torch.repeat_interleave(torch.arange(p.n_points, device=p.indptr.device), p.indptr[1:] - p.indptr[:-1])
        return torch.stack([rows, p.indices.long()], 0)

    def forward(self, *args):
        raise NotImplementedError("subclass ElementAssembler and define forward(...)")

    def _resolve_form(self, fn, element_data, point_data, scalar_data) -> F_.BilinearForm:
        cls_forward = type(self).forward
        if fn is None and self._builtin_form is not None and cls_forward is self._builtin_forward_impl():
            return self._builtin_form_instance()
        fn = self.forward if fn is None else fn
        key = (fn.__func__ if hasattr(fn, "__func__") else fn, tuple(sorted(element_data)), tuple(sorted(point_data)),
               tuple(sorted(scalar_data)))
        if key not in self._form_cache:
            params = list(inspect.signature(fn).parameters)
            known = {"u", "v", "gradu", "gradv"} | set(element_data) | set(point_data) | set(scalar_data)
            for p in params:
                if p not in known:
                    raise ValueError(f"{p} is not supported, please use `u`, `v`, `gradu`, `gradv` or more keys "
                                     f"provided by point_data, element_data or scalar_data")
            self._form_cache[key] = F_.recognise_bilinear(
                fn, self.topology.dim, set(element_data) | set(point_data) | set(scalar_data))
        return self._form_cache[key]

    @classmethod
    def _builtin_forward_impl(cls):
        return None

    def _builtin_form_instance(self):
        return self._builtin_form

    def __call__(self, points: Optional[torch.Tensor] = None, func: Optional[Callable] = None,
                 point_data: Optional[Mapping[str, torch.Tensor]] = None,
                 element_data: Optional[Mapping] = None,
                 scalar_data: Optional[Mapping] = None, batch_size: int = -1) -> SparseMatrix:
        assert isinstance(point_data, dict) or point_data is None, \
            f"point_data should be a dict, but got {type(point_data)}"
        topo = self.topology
        point_data = dict(point_data or {})
        element_data = dict(element_data or {})
        for k, v in list(element_data.items()):
            if isinstance(v, dict):
                assert len(v) == 1 and topo.element_type in v
                element_data[k] = v[topo.element_type]
            assert element_data[k].shape[0] == topo.n_elements, \
                f"the shape of {k} should be [{topo.n_elements}, ...], but got {element_data[k].shape[0]}"
        scalar_data = dict(scalar_data or {})
        if points is None:
            points = self.points
        assert points.shape[1] == topo.dim, f"the dimension of points should be {topo.dim}, but got {points.shape[1]}"
        assert points.shape[0] == topo.n_points
        for k, v in point_data.items():
            assert v.shape[0] == points.shape[0], f"the shape of {k} should be [n_point, ...], but got {v.shape}"
        _require_cuda(points, "points")
        form = self._resolve_form(func, element_data, point_data, scalar_data)
        from .autodiff import assemble_matrix
        return assemble_matrix(self, form, points, element_data, point_data, scalar_data)


def _autotune_assembler(asm, call, dtype, budgets, reps, use_cache):
    from . import autotune as AT
    dev = asm.points.device
    key = (f"assemble|{torch.cuda.get_device_name(dev)}|{asm.topology.element_type}|{type(asm).__name__}|"
           f"{dtype}|{asm.topology.n_elements}|{asm.topology.n_points}|q{asm.quadrature_order}")
    if use_cache:
        hit = AT.load_cache().get(key)
        if hit:
            asm.slot_budget = hit["slot_budget"]
            return hit

    def run(bgt):
        asm.slot_budget = bgt
        call()
    best, table = AT.pick(budgets, run, reps=reps)
    asm.slot_budget = best
    res = {"slot_budget": best, "table": table}
    if use_cache:
        AT.store_cache(key, res)
    return res


def _assembler_autotune(self, points=None, element_data=None, point_data=None, scalar_data=None,
                        budgets=(512, 1024, 2048, 4096, 6144), reps: int = 3, use_cache: bool = True) -> dict:
    """Pick the patch size (accumulator budget per patch) that assembles
    fastest for these inputs on this GPU; the choice is cached as JSON."""
    pts = self.points if points is None else points
    return _autotune_assembler(self, lambda: self(pts, element_data=element_data, point_data=point_data,
                                                  scalar_data=scalar_data), pts.dtype, budgets, reps, use_cache)


ElementAssembler.autotune = _assembler_autotune


class LaplaceElementAssembler(ElementAssembler):
    """K_ij = int grad N_i . grad N_j (assemble/builtin.py:25-63)."""
    _builtin_form = F_.BilinearForm("laplace", None)

    def forward(self, gradu, gradv):
        return gradu @ gradv

    @classmethod
    def _builtin_forward_impl(cls):
        return LaplaceElementAssembler.forward


class MassElementAssembler(ElementAssembler):
    """M_ij = int N_i N_j (assemble/builtin.py:65-101)."""
    _builtin_form = F_.BilinearForm("mass", None)

    def forward(self, u, v):
        return u * v

    @classmethod
    def _builtin_forward_impl(cls):
        return MassElementAssembler.forward


class LinearElasticityElementAssembler(ElementAssembler):
    """K_ij = int B_i^T C(E, nu) B_j (assemble/builtin.py:103-179); Voigt rows
    [xx, yy, zz, yz, xz, xy] (functional/elasticity.py:132-284)."""

    def __post_init__(self, E=1.0, nu=0.3):
        self.E = E
        self.nu = nu

    def forward(self, gradu, gradv):
        lam, mu = F_.reference_lame(float(self.E), float(self.nu))
        return F_.elasticity_block(gradu, gradv, lam, mu)

    @classmethod
    def _builtin_forward_impl(cls):
        return LinearElasticityElementAssembler.forward

    def _builtin_form_instance(self):
        lam, mu = F_.reference_lame(float(self.E), float(self.nu))
        return F_.BilinearForm("elasticity", None, 1.0, lam, mu)

    _builtin_form = F_.BilinearForm("elasticity", None)


class NodeAssembler(_AssemblerDevice, nn.Module):
    """Assemble a linear form into a node vector on the GPU."""

    precision = "emulated"

    def __init__(self, topology: MeshTopology, points: torch.Tensor, quadrature_order: int, *args, **kwargs):
        super().__init__()
        self.topology = topology
        self.quadrature_order = int(quadrature_order)
        self.register_buffer("points", points, persistent=False)
        self.element_types = [topology.element_type]
        self.n_points = topology.n_points
        self._form_cache = {}
        self.__post_init__(*args, **kwargs)

    def __post_init__(self, *args, **kwargs):
        pass

    @classmethod
    def from_mesh(cls, mesh, quadrature_order: int = 2, project: str = "reduce", *args, **kwargs):
        etype, elements = _mesh_single_type(mesh)
        topo = topology_for(elements.to(mesh.points.device), mesh.points, etype)
        return cls(topo, mesh.points, quadrature_order, *args, **kwargs)

    @classmethod
    def from_elements(cls, points: torch.Tensor, elements: Dict[str, torch.Tensor], quadrature_order: int = 2,
                      device="cpu", dtype=torch.float32, project: str = "reduce", *args, **kwargs):
        assert len(elements) == 1, "mixed element types are not on the GPU path"
        (etype, el), = elements.items()
        points = points.to(device=device, dtype=dtype)
        topo = topology_for(el.to(points.device), points, etype)
        return cls(topo, points, quadrature_order, *args, **kwargs)

    @classmethod
    def from_assembler(cls, obj, *args, **kwargs):
        assert isinstance(obj, (NodeAssembler, ElementAssembler))
        return cls(obj.topology, obj.points, obj.quadrature_order, *args, **kwargs)

    def forward(self, *args):
        raise NotImplementedError("subclass NodeAssembler and define forward(...)")

    # The reference's fast mode (assemble/node_assembler.py:416-536) swaps its
    # vmap path for broadcast operations, optionally under torch.compile.  The
    # load here is always one fused kernel launch, so these switches only
    # record the request; ``compile`` never calls torch.compile.
    def compile(self, mode: str = "disable", fullgraph: bool = False, dynamic=None, backend: str = "inductor",
                **kwargs) -> "NodeAssembler":
        """Accepted for drop-in use; returns ``self`` (the kernel path is already the fast path)."""
        self._compile_request = dict(mode=mode, fullgraph=fullgraph, dynamic=dynamic, backend=backend, **kwargs)
        return self

    def flat_mode(self) -> "NodeAssembler":
        return self.compile(mode="disable")

    def reset_compile(self) -> "NodeAssembler":
        self._compile_request = None
        return self

    def is_compiled(self) -> bool:
        return getattr(self, "_compile_request", None) is not None

    def _resolve_form(self, fn, point_data, scalar_data) -> F_.LinearForm:
        fn = self.forward if fn is None else fn
        key = (fn.__func__ if hasattr(fn, "__func__") else fn, tuple(sorted(point_data)), tuple(sorted(scalar_data)))
        if key not in self._form_cache:
            builtin = getattr(self, "_linear_form", None)
            if builtin is not None and fn == self.forward and type(self).forward is getattr(self, "_builtin_forward"):
                self._form_cache[key] = builtin()
            else:
                self._form_cache[key] = F_.recognise_linear(fn, self.topology.dim, set(point_data), set(scalar_data))
        return self._form_cache[key]

    def __call__(self, points: Optional[torch.Tensor] = None, func: Optional[Callable] = None,
                 point_data: Optional[Dict[str, torch.Tensor]] = None,
                 scalar_data: Optional[Dict[str, torch.Tensor]] = None, batch_size: int = 1) -> torch.Tensor:
        topo = self.topology
        point_data = dict(point_data or {})
        scalar_data = dict(scalar_data or {})
        if points is None:
            points = self.points
        assert points.shape[1] == topo.dim, f"the dimension of the points should be {topo.dim}, but got {points.shape[1]}"
        for k, v in point_data.items():
            assert v.shape[0] == points.shape[0], f"the shape of {k} should be [n_point, ...], but got {v.shape}"
        _require_cuda(points, "points")
        form = self._resolve_form(func, point_data, scalar_data)
        from .autodiff import assemble_load
        return assemble_load(self, form, points, point_data, scalar_data)


def const_node_assembler(c=1):
    """NodeAssembler subclass for f_i = int c N_i (assemble/builtin.py:886-927)."""

    class ConstNodeAssembler(NodeAssembler):
        def __post_init__(self, c=c):
            self.c = c

        def forward(self, v):
            return self.c * v

        def _linear_form(self):
            cc = torch.as_tensor(self.c, dtype=torch.float64).reshape(-1).cpu()
            return F_.LinearForm("const", const=cc, n_comp=int(cc.numel()))

    ConstNodeAssembler._builtin_forward = ConstNodeAssembler.forward
    return ConstNodeAssembler


def func_node_assembler(f=lambda x: x):
    """NodeAssembler subclass for f_i = int f(x) N_i (assemble/builtin.py:929-969)."""

    class FuncNodeAssembler(NodeAssembler):
        def __post_init__(self, f=f):
            self.f = f

        def forward(self, x, v):
            return self.f(x) * v

        def _linear_form(self):
            return F_.LinearForm("func", func=self.f, n_comp=1)

    FuncNodeAssembler._builtin_forward = FuncNodeAssembler.forward
    return FuncNodeAssembler


def __getattr__(name):
    # NeoHookeanModel lives in energy.py (it subclasses ElementAssembler)
    if name == "NeoHookeanModel":
        from .energy import NeoHookeanModel
        return NeoHookeanModel
    raise AttributeError(name)
