"""Differentiable FDTD: receiver traces and their gradients with respect to per-cell relative
permittivity and conductivity, through a hand-written discrete adjoint on the GPU.

The reference has no gradient path; this module adds one for gprMax models of the kind the
time loop runs (3D, non-dispersive, CFS PML of HORIPML order 1, Hertzian dipoles, field
receivers). The model it differentiates is the reference's update with per-cell materials:

* each cell has its own eps_r and sigma (mu_r = 1, no magnetic loss); an E edge takes the
  arithmetic mean of the four cells around it, as the reference's dielectric smoothing does
  for averaged materials (``materials.py:process_materials`` / ``yee_cell_build_ext.pyx``);
* E edges: CA = (eps/dt - sigma/2) / (eps/dt + sigma/2), CB = 1 / (eps/dt + sigma/2)
  (``materials.py:calculate_update_coeffsE``); the curl term uses CB/d and the PML and source
  terms use CB (the coefficient table's column 4); edges the reference never updates keep
  CA = 1, CB = 0;
* H nodes: DA = 1, DB = dt/mu0, curl term DB/d (``calculate_update_coeffsH``);
* the update, ranges, PML slab corrections (``pml_updates_*_HORIPML_ext.pyx`` order 1) and
  Hertzian-dipole injection (``sources.py:163-193``) of the reference; receivers sample one E
  component at the start of every iteration (``fields_outputs.py:40-67``).

``FDTDTraces`` is the ``torch.autograd.Function``: forward runs the time loop on the GPU
(``gbf_adj_forward``) and keeps a checkpoint at the start of every segment; backward runs the
transposed (reverse-time) updates (``gbf_adj_backward``), recomputing each segment's states
from its checkpoint, and returns dL/dCA and dL/dCB per edge, accumulated in fp64. By default
(``checkpoint_interval=-1``) the last segment is as long as 60 % of the free device memory can
hold and the forward leaves its states in place, so only the steps before it are recomputed
(none when the whole run fits); ``checkpoint_interval=0`` gives segments of ceil(sqrt(T))
steps. The map
from (eps_r, sigma) to (CA, CB) is plain torch, so autograd carries the gradient to the cells.
"""
import ctypes

import numpy as np

from . import _native
from .constants import e0, m0
from .exceptions import SolverError

PML_SLABS = ['x0', 'y0', 'z0', 'xmax', 'ymax', 'zmax']
COMPONENTS = {'Ex': 0, 'Ey': 1, 'Ez': 2}


class AdjointModel:
    """The fixed part of a differentiable model, built from gprMax input lines by this
    package's front-end: grid, dt and iterations, PML profile rows, dipole sources with their
    waveform tables, receivers (component, node). Materials in the input are ignored; the
    per-cell eps_r and sigma are the differentiable parameters."""

    def __init__(self, lines, receiver_component='Ez'):
        from .model import build_grid
        G = build_grid(lines, messages=False)
        if G.nx < 2 or G.ny < 2 or G.nz < 2:
            raise SolverError('the adjoint solver handles 3D grids only')
        if not (np.float32(G.dx) == np.float32(G.dy) == np.float32(G.dz)):
            raise SolverError('the adjoint solver needs cubic cells (dx = dy = dz)')
        if G.pmls and (G.pmlformulation != 'HORIPML' or len(G.cfs) != 1):
            raise SolverError('the adjoint solver supports HORIPML with one CFS term')
        if G.voltagesources or G.magneticdipoles or getattr(G, 'transmissionlines', None):
            raise SolverError('the adjoint solver supports Hertzian dipoles only')
        self.G = G
        self.nx, self.ny, self.nz = G.nx, G.ny, G.nz
        self.iterations = G.iterations
        self.d = float(G.dx)
        self.dt = float(G.dt)
        self.thickness = [0] * 6
        self.pml_rows = {}
        for pml in G.pmls:
            s = PML_SLABS.index(pml.ID)
            self.thickness[s] = pml.thickness
            self.pml_rows[s] = [np.ascontiguousarray(getattr(pml, n)[0], dtype=np.float32)
                                for n in ('ERA', 'ERB', 'ERE', 'ERF', 'HRA', 'HRB', 'HRE', 'HRF')]
        # H coefficients of free space (mu_r = 1, sigma* = 0), in fp32 as the reference stores
        DB = self.dt / m0
        self.dbd = float(np.float32(DB / self.d))
        self.srcm = float(np.float32(DB))
        from .sources import active_range
        self.sources = []
        for h in G.hertziandipoles:
            comp = 'xyz'.index(h.polarisation)
            first, last = active_range(h, G)
            wave = np.zeros(G.iterations, dtype=np.float32)
            if last >= first:
                wave[first:last + 1] = h.waveformvalues_wholestep[first:last + 1]
            scale = float(np.float32(h.dl) * np.float32(1 / (G.dx * G.dy * G.dz)))
            self.sources.append((comp, h.xcoord, h.ycoord, h.zcoord, scale, wave))
        self.receivers = []
        comp = COMPONENTS[receiver_component]
        for r in G.rxs:
            self.receivers.append((comp, r.xcoord, r.ycoord, r.zcoord))
        if not self.receivers:
            raise SolverError('the adjoint model needs at least one receiver')

    @property
    def shape(self):
        return (self.nx + 1, self.ny + 1, self.nz + 1)

    def edge_coefficients(self, eps_r, sigma):
        """Per-edge (CA, CB) as torch tensors [3][nx+1][ny+1][nz+1] from per-cell eps_r and
        sigma [nx][ny][nz] (differentiable; the dtype of the inputs)."""
        import torch
        nx, ny, nz = self.nx, self.ny, self.nz
        eps = eps_r * e0
        dt = self.dt
        CA = torch.ones((3,) + self.shape, dtype=eps_r.dtype, device=eps_r.device)
        CB = torch.zeros((3,) + self.shape, dtype=eps_r.dtype, device=eps_r.device)

        def avg4(a, comp):
            # mean of the four cells around the updated edges of component comp
            if comp == 0:    # Ex at (i, j, k), j in [1, ny), k in [1, nz)
                return 0.25 * (a[:, 1:, 1:] + a[:, :-1, 1:] + a[:, 1:, :-1] + a[:, :-1, :-1])
            if comp == 1:    # Ey: i in [1, nx), k in [1, nz)
                return 0.25 * (a[1:, :, 1:] + a[:-1, :, 1:] + a[1:, :, :-1] + a[:-1, :, :-1])
            return 0.25 * (a[1:, 1:, :] + a[:-1, 1:, :] + a[1:, :-1, :] + a[:-1, :-1, :])

        CA_parts, CB_parts = [], []
        for comp in range(3):
            e = avg4(eps, comp)
            s = avg4(sigma, comp)
            EA = e / dt + 0.5 * s
            EB = e / dt - 0.5 * s
            CA_parts.append(EB / EA)
            CB_parts.append(1 / EA)
        CA[0, :nx, 1:ny, 1:nz] = CA_parts[0]
        CB[0, :nx, 1:ny, 1:nz] = CB_parts[0]
        CA[1, 1:nx, :ny, 1:nz] = CA_parts[1]
        CB[1, 1:nx, :ny, 1:nz] = CB_parts[1]
        CA[2, 1:nx, 1:ny, :nz] = CA_parts[2]
        CB[2, 1:nx, 1:ny, :nz] = CB_parts[2]
        return CA, CB


class AdjointSolver:
    """GPU forward/adjoint engine of one ``AdjointModel`` (``gbf_adj_*`` in the C ABI)."""

    def __init__(self, model, checkpoint_interval=-1):
        """checkpoint_interval: steps per segment; 0: ceil(sqrt(iterations)); -1: the last
        segment sized to the free device memory (see the module docstring)."""
        self.model = model
        self.lib = _native.lib()
        self.h = ctypes.c_void_p(0)
        d = _native.AdjDesc()
        d.nx, d.ny, d.nz = model.nx, model.ny, model.nz
        d.iterations = model.iterations
        d.d = np.float32(model.d)
        d.dt = np.float32(model.dt)
        d.dbd = np.float32(model.dbd)
        d.srcm = np.float32(model.srcm)
        for s in range(6):
            d.pml_thickness[s] = model.thickness[s]
        d.nsrc = len(model.sources)
        d.nrx = len(model.receivers)
        d.checkpoint_interval = int(checkpoint_interval)
        self._check(self.lib.gbf_adj_create(ctypes.byref(d), ctypes.byref(self.h)), created=False)
        try:
            for s, rows in model.pml_rows.items():
                arr = (ctypes.c_void_p * 8)(*[r.ctypes.data for r in rows])
                self._check(self.lib.gbf_adj_upload_pml(self.h, s, arr))
            if model.sources:
                info = np.array([[c, i, j, k] for c, i, j, k, _, _ in model.sources], np.int32)
                scale = np.array([sc for _, _, _, _, sc, _ in model.sources], np.float32)
                waves = np.ascontiguousarray(np.stack([w for *_, w in model.sources]), np.float32)
                self._check(self.lib.gbf_adj_upload_sources(
                    self.h, info.ctypes.data, scale.ctypes.data, waves.ctypes.data))
            rx = np.array(model.receivers, np.int32)
            self._check(self.lib.gbf_adj_set_receivers(self.h, rx.ctypes.data))
        except Exception:
            self.close()
            raise

    def _check(self, rc, created=True):
        if rc != 0:
            buf = ctypes.create_string_buffer(1024)
            self.lib.gbf_adj_last_error(self.h if created else None, buf, 1024)
            raise SolverError('libgbfdtd adjoint error {}: {}'.format(rc, buf.value.decode()))

    def forward(self, CA, CB):
        """fp32 CUDA tensors CA, CB [3][nx+1][ny+1][nz+1] -> traces [nrx][iterations]."""
        import torch
        m = self.model
        traces = torch.empty((len(m.receivers), m.iterations), dtype=torch.float32, device=CA.device)
        torch.cuda.current_stream(CA.device).synchronize()
        self._check(self.lib.gbf_adj_forward(self.h, CA.data_ptr(), CB.data_ptr(), traces.data_ptr()))
        return traces

    def backward(self, CA, CB, gtraces):
        """d(misfit)/d(CA, CB) in fp64 given d(misfit)/d(traces) (fp32 CUDA tensors); needs the
        checkpoints of the last ``forward`` with the same CA, CB."""
        import torch
        gCA = torch.empty((3,) + self.model.shape, dtype=torch.float64, device=CA.device)
        gCB = torch.empty_like(gCA)
        torch.cuda.current_stream(CA.device).synchronize()
        self._check(self.lib.gbf_adj_backward(self.h, CA.data_ptr(), CB.data_ptr(),
                                              gtraces.data_ptr(), gCA.data_ptr(), gCB.data_ptr()))
        return gCA, gCB

    def close(self):
        if self.h and self.h.value:
            self.lib.gbf_adj_destroy(self.h)
        self.h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _traces_function():
    import torch

    class FDTDTraces(torch.autograd.Function):
        """traces = FDTDTraces.apply(CA, CB, solver): the GPU time loop as a differentiable
        function of the per-edge coefficients; backward is the checkpointed discrete adjoint."""

        @staticmethod
        def forward(ctx, CA, CB, solver):
            CA32 = CA.detach().to(device='cuda', dtype=torch.float32).contiguous()
            CB32 = CB.detach().to(device='cuda', dtype=torch.float32).contiguous()
            traces = solver.forward(CA32, CB32)
            ctx.save_for_backward(CA32, CB32)
            ctx.solver = solver
            ctx.dtypes = (CA.dtype, CB.dtype, CA.device)
            return traces

        @staticmethod
        def backward(ctx, gtraces):
            CA32, CB32 = ctx.saved_tensors
            g = gtraces.detach().to(torch.float32).contiguous()
            gCA, gCB = ctx.solver.backward(CA32, CB32, g)
            ta, tb, dev = ctx.dtypes
            return gCA.to(device=dev, dtype=ta), gCB.to(device=dev, dtype=tb), None

    return FDTDTraces


_FDTD_TRACES = None


def fdtd_traces(CA, CB, solver):
    """Differentiable receiver traces [nrx][iterations] for per-edge CA, CB."""
    global _FDTD_TRACES
    if _FDTD_TRACES is None:
        _FDTD_TRACES = _traces_function()
    return _FDTD_TRACES.apply(CA, CB, solver)


def misfit(model, solver, eps_r, sigma, observed):
    """0.5 * sum((traces - observed)^2) in fp64 for per-cell eps_r, sigma (torch tensors on the
    GPU); differentiable with respect to eps_r and sigma."""
    import torch
    CA, CB = model.edge_coefficients(eps_r, sigma)
    traces = fdtd_traces(CA, CB, solver)
    return 0.5 * ((traces.to(torch.float64) - observed.to(torch.float64)) ** 2).sum(), traces
