"""Batched stepping of thousands of independent instances of uneven size.

A :class:`BatchedSolver` wraps one ``shk_plan`` of ``libshocks.so``: a packed
device buffer of all instances' interior cells (``offsets[B+1]``), per-instance
``dx``, CFL constant, time, final time and dt history, stepped by a persistent
kernel that fuses the three SSPRK33 stages, computes the next step's CFL dt on
the device and never returns to the host between steps. It is the batched form
of ``step()`` (``src/pyshocks/timestepping.py:89-152``) with the Rusanov CFL
estimate (``src/pyshocks/burgers/schemes.py:121-127``).
"""

from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np
import torch

from pyshocks_gb300 import _lib as L

_DTYPES = {torch.float64: L.SHK_F64, torch.float32: L.SHK_F32}


def partition_instances(sizes: Sequence[int], world: int, work_per_cell: Sequence[float] | None = None):
    """Longest-processing-time assignment of independent instances to *world*
    ranks (instances never couple, so ranks need no data-path collective).
    Returns one sorted index array per rank; the cost of an instance is its
    cell count (times *work_per_cell*, e.g. its step count, when given)."""
    sizes = np.asarray(sizes, dtype=np.float64)
    cost = sizes * (np.asarray(work_per_cell, dtype=np.float64) if work_per_cell is not None else 1.0)
    order = np.argsort(-cost, kind="stable")
    load = np.zeros(world)
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(load))
        parts[r].append(int(i))
        load[r] += cost[i]
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def pack_offsets(sizes: Sequence[int]) -> np.ndarray:
    """``offsets[B+1]`` of a contiguous packing of instances of *sizes* cells."""
    off = np.zeros(len(sizes) + 1, dtype=np.int64)
    off[1:] = np.cumsum(np.asarray(sizes, dtype=np.int64))
    return off


def _boundary_tables(B: int, device, left: str, right: str | None, dirichlet, neumann):
    """Boundary kinds and the ``(B, 2, 3)`` Dirichlet / ``(B, 2)`` Neumann
    tables (float64 on *device*) of :meth:`BatchedSolver.set_boundary`."""
    kinds = {"periodic": L.SHK_BC_PERIODIC, "dirichlet": L.SHK_BC_DIRICHLET,
             "neumann": L.SHK_BC_NEUMANN}
    right = left if right is None else right

    def table(v, shape):
        if v is None:
            return None
        t = torch.as_tensor(v, dtype=torch.float64, device=device)
        if t.dim() == 1 and t.numel() == 2:
            t = t.reshape((1, 2) + (1,) * (len(shape) - 2)).expand((B,) + shape[1:])
        return t.reshape(shape).contiguous()

    return kinds[left], kinds[right], table(dirichlet, (B, 2, 3)), table(neumann, (B, 2))


class HostStepper:
    """A batch whose state lives in host memory (``shk_host_stepper``).

    :meth:`advance` copies the packed host state in, takes ``nsteps`` CFL
    steps from t = 0 and copies the result out, with the batch split by
    instance into *chunks* pipelined over copy and compute streams: the copies
    of one chunk overlap the steps of the others. The result is bit-identical
    to a :class:`BatchedSolver` over the whole batch. Host tensors should be
    pinned (``pin_memory()``) for the copies to overlap.
    """

    def __init__(self, scheme, sizes: Sequence[int], dx: float | Sequence[float], *,
                 theta: float = 1.0, dtype: torch.dtype = torch.float64, tile: int = 0,
                 ctas_per_sm: int = 0, chunks: int = 0):
        if dtype not in _DTYPES:
            raise TypeError(f"unsupported dtype {dtype}")
        self.lib = L.lib()
        self.sizes = np.asarray(sizes, dtype=np.int64)
        self.B = int(self.sizes.size)
        self.offsets = pack_offsets(self.sizes)
        self.total = int(self.offsets[-1])
        self.dtype = dtype
        dxs = np.broadcast_to(np.asarray(dx, dtype=np.float64), (self.B,)).copy()
        self.cfl = np.array([scheme.cfl_constant(float(h)) for h in dxs], dtype=np.float64)
        cs = scheme.c_scheme(float(dxs[0]))
        opts = L.ShkPlanOpts(dtype=_DTYPES[dtype], tile=int(tile), max_steps=0,
                             ctas_per_sm=int(ctas_per_sm))
        hs = ctypes.c_void_p()
        L.check(self.lib.shk_host_stepper_create(cs, self.B, self.offsets.ctypes.data,
                                                 dxs.ctypes.data, self.cfl.ctypes.data,
                                                 float(theta), ctypes.byref(opts), int(chunks),
                                                 ctypes.byref(hs)), "host_stepper_create")
        self._hs = hs
        self.chunks = int(self.lib.shk_host_stepper_num_chunks(hs))

    def __del__(self):
        hs = getattr(self, "_hs", None)
        if hs is not None and hs.value:
            try:
                torch.cuda.synchronize()
                self.lib.shk_host_stepper_destroy(hs)
            except Exception:
                pass
            self._hs = None

    def advance(self, u_in: torch.Tensor, u_out: torch.Tensor | None = None,
                nsteps: int = 1) -> torch.Tensor:
        """``u_out`` = ``u_in`` advanced by *nsteps* steps (CPU tensors of the
        stepper's dtype, packed layout; ``u_out`` may be ``u_in``). The call
        does not block: ``u_out`` holds the result once the current stream has
        passed it (``torch.cuda.current_stream().synchronize()``)."""
        for t in (u_in,) if u_out is None else (u_in, u_out):
            if t.device.type != "cpu" or t.dtype != self.dtype or not t.is_contiguous() \
                    or t.numel() != self.total:
                raise ValueError("host state must be a contiguous CPU tensor of the "
                                 "stepper's dtype and packed size")
        if u_out is None:
            u_out = torch.empty(u_in.shape, dtype=self.dtype, pin_memory=u_in.is_pinned())
        L.check(self.lib.shk_host_stepper_advance(self._hs, u_in.data_ptr(), u_out.data_ptr(),
                                                  int(nsteps), L.stream_handle()),
                "host_stepper_advance")
        return u_out

    def set_boundary(self, left: str = "periodic", right: str | None = None, *,
                     dirichlet=None, neumann=None) -> None:
        """As :meth:`BatchedSolver.set_boundary`, for every chunk."""
        lk, rk, d, nm = _boundary_tables(self.B, torch.device("cuda"), left, right, dirichlet,
                                         neumann)
        L.check(self.lib.shk_host_stepper_set_boundary(self._hs, lk, rk, L.ptr(d), L.ptr(nm),
                                                       L.stream_handle()),
                "host_stepper_set_boundary")
        self._bc_keep = (d, nm)

    def status(self) -> int:
        st = ctypes.c_int32()
        L.check(self.lib.shk_host_stepper_status(self._hs, ctypes.byref(st), L.stream_handle()))
        return int(st.value)


class BatchedSolver:
    """Persistent batched SSPRK33 solver for one scheme on periodic domains.

    :arg scheme: a scheme of :mod:`pyshocks_gb300.burgers`. The global
        Lax-Friedrichs flux (WENO-JS5, float64, periodic instances) steps with
        one launch per stage instead of the fused kernel: its wave speed is the
        per-stage maximum over the whole instance.
    :arg sizes: number of interior cells of every instance.
    :arg dx: cell size per instance (or a scalar).
    :arg theta: Courant factor of the driver closure ``theta * predict_timestep``.
    :arg dtype: ``torch.float64`` or ``torch.float32`` state.
    :arg max_steps: capacity of the per-step dt history (for the adjoint).
    :arg tile: cells per work item (0: the library default, which depends on
        the scheme, precision and whether the plan keeps a dt history; ``"auto"``:
        chosen with ``ctas_per_sm`` by :func:`pyshocks_gb300.autotune.tune`).
    :arg ctas_per_sm: resident CTAs per SM of the persistent grid (0: as many
        as the shared memory allows, at most 8).
    """

    def __init__(
        self,
        scheme,
        sizes: Sequence[int],
        dx: float | Sequence[float],
        *,
        theta: float = 1.0,
        dtype: torch.dtype = torch.float64,
        tile: int | str = 0,
        max_steps: int = 0,
        ctas_per_sm: int = 0,
        device: str | torch.device = "cuda",
    ):
        if dtype not in _DTYPES:
            raise TypeError(f"unsupported dtype {dtype}")
        self.lib = L.lib()
        self.scheme = scheme
        self.sizes = np.asarray(sizes, dtype=np.int64)
        self.B = int(self.sizes.size)
        self.offsets = pack_offsets(self.sizes)
        self.total = int(self.offsets[-1])
        dxs = np.broadcast_to(np.asarray(dx, dtype=np.float64), (self.B,)).copy()
        self.dx = dxs
        self.cfl = np.array([scheme.cfl_constant(float(h)) for h in dxs], dtype=np.float64)
        nu_for = getattr(scheme, "nu_for", None)
        if nu_for is not None and len({nu_for(float(h)) for h in np.unique(dxs)}) > 1:
            # Rusanov(alpha != 1): nu = dx^(alpha - 1) (scalar.py:231-234)
            raise ValueError("the scheme's dissipation depends on dx and a plan takes one "
                             "value: instances of Rusanov(alpha != 1) must share dx")
        self.theta = float(theta)
        self.dtype = dtype
        self.device = torch.device(device)
        self.max_steps = int(max_steps)
        self._cs = scheme.c_scheme(float(dxs[0]))
        if tile == "auto":
            from pyshocks_gb300 import autotune

            best = autotune.tune(scheme, self.sizes, dxs, dtype=dtype, theta=theta,
                                 device=self.device, adjoint=self.max_steps > 0)
            tile, ctas_per_sm = best.tile, best.ctas_per_sm
        self.tile = int(tile)
        self.ctas_per_sm = int(ctas_per_sm)
        opts = L.ShkPlanOpts(dtype=_DTYPES[dtype], tile=int(tile), max_steps=self.max_steps,
                             ctas_per_sm=int(ctas_per_sm))
        plan = ctypes.c_void_p()
        L.check(
            self.lib.shk_plan_create(
                self._cs, self.B, self.offsets.ctypes.data, dxs.ctypes.data,
                self.cfl.ctypes.data, self.theta, ctypes.byref(opts), ctypes.byref(plan)),
            "plan_create",
        )
        self._plan = plan
        self.buf_a = torch.zeros(self.total, dtype=dtype, device=self.device)
        self.buf_b = torch.zeros(self.total, dtype=dtype, device=self.device)
        self._steps = 0

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and plan.value:
            try:
                torch.cuda.synchronize()
                self.lib.shk_plan_destroy(plan)
            except Exception:
                pass
            self._plan = None

    # {{{ state

    @property
    def u(self) -> torch.Tensor:
        """Packed current state (a view of the solver's buffer)."""
        return self.buf_a if self._steps % 2 == 0 else self.buf_b

    @property
    def steps(self) -> int:
        return self._steps

    def instance(self, b: int, u: torch.Tensor | None = None) -> torch.Tensor:
        u = self.u if u is None else u
        return u[int(self.offsets[b]) : int(self.offsets[b + 1])]

    def time(self) -> torch.Tensor:
        """Per-instance time (a copy, float64)."""
        out = torch.empty(self.B, dtype=torch.float64, device=self.device)
        L.check(self.lib.shk_plan_copy_time(self._plan, out.data_ptr(), L.stream_handle()))
        return out

    def dt_history(self) -> torch.Tensor:
        """``(steps, B)`` time steps taken (0 for inactive instances)."""
        if not self.max_steps:
            raise RuntimeError("solver created with max_steps=0")
        n = min(self._steps, self.max_steps)
        out = torch.empty((self.max_steps, self.B), dtype=torch.float64, device=self.device)
        L.check(self.lib.shk_plan_copy_dt_history(self._plan, out.data_ptr(), L.stream_handle()))
        return out[:n]

    def status(self) -> int:
        st = ctypes.c_int32()
        L.check(self.lib.shk_plan_status(self._plan, ctypes.byref(st), L.stream_handle()))
        return int(st.value)

    def check_status(self) -> None:
        """Raise on the plan's device status bits: a non-finite time step
        (``ValueError``, as ``step()``), an expired bounded wait, or (in the
        bounds-check build) an index outside its array (``RuntimeError``). A
        launch that reported either of the latter leaves its output undefined;
        reset the plan before stepping it again."""
        st = self.status()
        if st & L.ERR_NONFINITE:
            raise ValueError("Time step is not finite (an instance was frozen)")
        if st & L.ERR_TIMEOUT:
            raise RuntimeError("bounded device wait expired in the step kernel")
        if st & L.ERR_BOUNDS:
            raise RuntimeError("a kernel index left its array (bounds-check build)")

    # }}}

    def reset(self, u0: torch.Tensor, *, t0=None, tfinal=None) -> None:
        """Load the packed initial state (any device/dtype) and reset time.
        *tfinal* ``None`` means no final time (the reference's ``finfo.max``)."""
        self.buf_a.copy_(u0.reshape(-1).to(self.buf_a))
        t0d = _per_instance(t0, self.B, self.device, 0.0)
        tfd = _per_instance(tfinal, self.B, self.device, float(np.finfo(np.float64).max))
        self._steps = 0
        L.check(
            self.lib.shk_plan_reset(self._plan, self.buf_a.data_ptr(), t0d.data_ptr(),
                                    tfd.data_ptr(), L.stream_handle()),
            "plan_reset",
        )
        self._keep = (t0d, tfd)

    def set_boundary(self, left: str = "periodic", right: str | None = None, *,
                     dirichlet=None, neumann=None) -> None:
        """Time-independent boundaries of every instance (``"periodic"``,
        ``"dirichlet"`` or ``"neumann"`` per side; periodic on both sides or
        on neither). *dirichlet*: ghost values ``(B, 2, 3)`` (side, then the
        ghost next to the interior first), or ``(2,)`` per side for all
        ghosts and instances; *neumann*: gradients ``(B, 2)`` or ``(2,)``.
        The adjoint of such a plan is the exact transpose with the boundary
        data as constants."""
        lk, rk, d, nm = _boundary_tables(self.B, self.device, left, right, dirichlet, neumann)
        L.check(self.lib.shk_plan_set_boundary(self._plan, lk, rk, L.ptr(d), L.ptr(nm),
                                               L.stream_handle()), "plan_set_boundary")
        self._bc_keep = (d, nm)

    def set_boundary_steps(self, left: str, right: str | None = None, *, dirichlet=None,
                           neumann=None) -> None:
        """Time-dependent boundary data: *dirichlet* ``(nsteps, 3, B, 2, 3)``
        ghost values or *neumann* ``(nsteps, 3, B, 2)`` gradients at the stage
        times ``t, t + dt, t + dt/2`` of each step (steps past the table take
        its last row). The caller evaluates them at its stage times, so they
        go with prescribed steps (:meth:`set_fixed_dt`)."""
        kinds = {"periodic": L.SHK_BC_PERIODIC, "dirichlet": L.SHK_BC_DIRICHLET,
                 "neumann": L.SHK_BC_NEUMANN}
        right = left if right is None else right

        def table(v, tail):
            if v is None:
                return None
            t = torch.as_tensor(v, dtype=torch.float64, device=self.device).contiguous()
            if t.dim() != 3 + len(tail) or t.shape[1] != 3 or tuple(t.shape[2:]) != (self.B,) + tail:
                raise ValueError(f"expected (nsteps, 3, {self.B}, {', '.join(map(str, tail))}), "
                                 f"got {tuple(t.shape)}")
            return t

        d = table(dirichlet, (2, 3))
        nm = table(neumann, (2,))
        nsteps = (d if d is not None else nm).shape[0] if (d is not None or nm is not None) else 0
        L.check(self.lib.shk_plan_set_boundary_steps(self._plan, kinds[left], kinds[right], L.ptr(d),
                                                     L.ptr(nm), int(nsteps), L.stream_handle()),
                "plan_set_boundary_steps")
        self._bc_keep = (d, nm)

    def set_fixed_dt(self, dt=None, nsteps: int | None = None) -> None:
        """Prescribe the time steps instead of the CFL step.

        *dt* is a ``(nsteps, B)`` table (e.g. a recorded :meth:`dt_history`,
        replayed exactly), a ``(nsteps,)`` sequence shared by all instances, or
        a scalar repeated *nsteps* times (the fixed step of
        :func:`~pyshocks_gb300.timestepping.predict_timestep_from_maxit`).
        Steps past the table, and steps ``<= 0``, leave an instance unchanged;
        the final time is not consulted. ``None`` returns to CFL steps.
        """
        if dt is None:
            L.check(self.lib.shk_plan_set_fixed_dt(self._plan, None, 0, L.stream_handle()),
                    "plan_set_fixed_dt")
            self._dt_fixed = None
            return
        t = torch.as_tensor(dt, dtype=torch.float64, device=self.device)
        if t.ndim == 0:
            if nsteps is None:
                raise ValueError("a scalar step needs nsteps")
            t = t.expand(int(nsteps), self.B)
        elif t.ndim == 1:
            t = t[:, None].expand(t.shape[0], self.B)
        if t.ndim != 2 or t.shape[1] != self.B:
            raise ValueError(f"expected a (nsteps, {self.B}) table, got {tuple(t.shape)}")
        t = t.contiguous()
        L.check(self.lib.shk_plan_set_fixed_dt(self._plan, t.data_ptr(), int(t.shape[0]),
                                               L.stream_handle()), "plan_set_fixed_dt")
        self._dt_fixed = t  # kept alive until the stream-ordered copy has run

    def step(self, nsteps: int = 1, *, graph: bool = False) -> torch.Tensor:
        """Advance all active instances by *nsteps* SSPRK33 steps."""
        stream = L.stream_handle()
        if graph and nsteps >= 2 and self._steps % 2 == 0 and stream != 0:
            n2 = nsteps - nsteps % 2
            L.check(self.lib.shk_plan_step_graph(self._plan, self.buf_a.data_ptr(),
                                                 self.buf_b.data_ptr(), n2, stream), "plan_step_graph")
            self._steps += n2
            nsteps -= n2
        if nsteps:
            L.check(self.lib.shk_plan_step(self._plan, self.buf_a.data_ptr(),
                                           self.buf_b.data_ptr(), nsteps, stream), "plan_step")
            self._steps += nsteps
        return self.u

    def reduce(self, p: int = 0, u: torch.Tensor | None = None) -> torch.Tensor:
        """Per-instance FP64 ``sum u`` (p=0), ``sum |u|`` (p=1), ``sum u^2``
        (p=2) or ``max |u|`` (p=-1), deterministic order."""
        u = self.u if u is None else u
        out = torch.empty(self.B, dtype=torch.float64, device=self.device)
        L.check(self.lib.shk_plan_reduce(self._plan, u.data_ptr(), int(p), out.data_ptr(),
                                         L.stream_handle()), "plan_reduce")
        return out

    def norm(self, p=1, u: torch.Tensor | None = None, *, weighted: bool = False) -> torch.Tensor:
        """Per-instance interior norms of ``src/pyshocks/grid.py:444-506`` (p = 1,
        2 or inf; ``weighted`` multiplies the sums by dx), from FP64 sums."""
        if p == 1:
            r = self.reduce(1, u)
        elif p == 2:
            r = self.reduce(2, u)
        elif p in {np.inf, "inf"}:
            return self.reduce(-1, u)
        else:
            raise ValueError(f"Unrecognized norm order 'p': {p!r}.")
        if weighted:
            r = r * torch.as_tensor(self.dx, device=r.device)
        return r if p == 1 else torch.sqrt(r)


def _per_instance(v, B, device, default) -> torch.Tensor:
    if v is None:
        return torch.full((B,), default, dtype=torch.float64, device=device)
    t = torch.as_tensor(v, dtype=torch.float64, device=device)
    if t.dim() == 0:
        t = t.expand(B)
    return t.contiguous().clone()

