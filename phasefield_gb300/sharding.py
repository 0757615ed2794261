"""One simulation sharded over ranks: slab decomposition of the cell lattice along its slowest
axis with one ghost cell layer per side, and a halo exchange of node planes after every block.

The reference distributes a simulation with deal.II's MPI partitioner: ghost values are
updated before each operator evaluation and interface contributions are reduce-added after it
(`update_ghost_values`, `compress`; src/core/group_solution_handler.cc:293-302,
src/solvers/mf_operator.cc:24). Here each rank instead computes one extra layer of cells on
each side of its slab, so every node it owns receives all of its cell contributions locally:
no reduce-add is needed, only ghost node values after a field changes. Vectors are in lattice
order with the split axis slowest, so a set of node planes is one contiguous range per
component and travels without packing. The exchange is the only collective of the data path
(NCCL on GPUs, gloo on CPUs), plus one logical-or of the non-finite flags per increment, as
`Problem::solve_increment` does (problem.cc:459-477).

Linear blocks (ShardedLinear): deal.II's SolverCG as LinearSolver::do_linear_solve runs it
(linear_solver.h:348-402), with every vector sharded like the fields. The operator apply of a
rank is complete on the rows it owns (its ghost cells contribute locally), so an apply needs
only the ghost planes of its input, refreshed by the same halo exchange; inner products sum
the owned rows of every rank and meet in one all-reduce of a float64 scalar
(linear_solver.h:357-379 reduces them over MPI the same way). Preconditioners: none, or the
reference's PreconditionerType::Chebyshev, whose diagonal is local and whose eigenvalue estimate
and inner applies use the same exchange and reductions; the multigrid hierarchy stays per GPU.

Scope: explicit, constant and post-processing blocks (the explicit increment loop), and single-
field Linear blocks with homogeneous Dirichlet values through ShardedLinear. Newton blocks are
rejected.
"""
from __future__ import annotations

import copy
import ctypes
from dataclasses import dataclass

import numpy as np

from .problem import Constant, Explicit, NucleationRate, PostProcess, Primary, RectangularMesh


@dataclass
class Slab:
    """The part of a global mesh one rank computes.

    Owned cells [c0, c1) along `axis`; `ghost_lo` / `ghost_hi` tell whether a ghost cell layer
    precedes / follows them (always with a neighbour or periodicity). Local node planes along the
    axis (k = degree): [0, k*ghost_lo) left ghosts, then the owned planes, then the right ghosts.
    """
    rank: int
    size: int
    axis: int
    degree: int
    n_cells: int          # global cells along the axis
    periodic: bool
    c0: int
    c1: int
    ghost_lo: int
    ghost_hi: int
    left: int | None      # neighbour ranks (None at a non-periodic end)
    right: int | None
    mesh: RectangularMesh  # the local mesh (ghost cells included)
    plane_size: int       # nodes per node plane (product over the other axes)

    @property
    def local_cells(self) -> int:
        return self.c1 - self.c0 + self.ghost_lo + self.ghost_hi

    @property
    def local_planes(self) -> int:
        return self.degree * self.local_cells + 1

    @property
    def n_nodes(self) -> int:
        return self.local_planes * self.plane_size

    def global_plane(self, local_plane: int) -> int:
        """Global plane of a local plane, periodic images folded onto their masters."""
        g = local_plane - self.degree * self.ghost_lo + self.degree * self.c0
        return g % (self.degree * self.n_cells) if self.periodic else g


    # planes this rank sends: to the left neighbour its first k+1 owned planes (the nodes of
    # the neighbour's right ghost cell), to the right neighbour its last k owned planes (the
    # neighbour's left ghost cell without the shared plane, which the neighbour owns)
    def send_left_planes(self) -> tuple[int, int]:
        k, lo = self.degree, self.degree * self.ghost_lo
        return lo, lo + k + 1

    def send_right_planes(self) -> tuple[int, int]:
        k, lo = self.degree, self.degree * self.ghost_lo
        end = lo + k * (self.c1 - self.c0)
        return end - k, end

    def recv_right_planes(self) -> tuple[int, int]:
        start = self.degree * (self.ghost_lo + self.c1 - self.c0)
        return start, start + self.degree + 1

    def recv_left_planes(self) -> tuple[int, int]:
        return 0, self.degree

    def owned_planes(self) -> tuple[int, int]:
        """Local planes whose values this rank contributes to the global vector."""
        lo = self.degree * self.ghost_lo
        hi = lo + self.degree * (self.c1 - self.c0)
        if not self.periodic and self.right is None:
            hi += 1  # the last plane of a non-periodic axis
        return lo, hi


def partition(mesh: RectangularMesh, rank: int, size: int) -> Slab:
    """Slab of `rank` among `size` ranks: cells along the slowest axis split as evenly as
    possible (at least 2 per rank)."""
    axis = mesh.dim - 1
    k = mesh.degree
    nc = mesh.cells[axis]
    if size > 1 and nc < 2 * size:
        raise ValueError(f"{nc} cells along the split axis cannot give {size} ranks 2 cells each")
    base, extra = divmod(nc, size)
    counts = [base + (1 if r < extra else 0) for r in range(size)]
    c0 = sum(counts[:rank])
    c1 = c0 + counts[rank]
    periodic = bool(mesh.periodic[axis])
    left = (rank - 1) % size if (rank > 0 or periodic) else None
    right = (rank + 1) % size if (rank < size - 1 or periodic) else None
    ghost_lo = 1 if left is not None else 0
    ghost_hi = 1 if right is not None else 0
    h = [mesh.size[d] / mesh.cells[d] for d in range(mesh.dim)]
    cells_local = list(mesh.cells)
    cells_local[axis] = c1 - c0 + ghost_lo + ghost_hi
    lower = list(mesh.lower) + [0.0] * (3 - len(mesh.lower))
    size_local = list(mesh.size)
    lower[axis] = mesh.lower[axis] + (c0 - ghost_lo) * h[axis]
    size_local[axis] = cells_local[axis] * h[axis]
    per = list(mesh.periodic) + [0] * (3 - len(mesh.periodic))
    per[axis] = 0  # the exchange carries the split axis' periodicity
    local = RectangularMesh(dim=mesh.dim, degree=k, size=tuple(size_local),
                            subdivisions=tuple(cells_local) + (1,) * (3 - mesh.dim), lower=tuple(lower),
                            global_refinement=0, periodic=tuple(per))
    plane = 1
    for d in range(mesh.dim - 1):
        plane *= mesh.nodes[d]
    return Slab(rank, size, axis, k, nc, periodic, c0, c1, ghost_lo, ghost_hi, left, right, local, plane)


def local_from_global(slab: Slab, v: np.ndarray, ncomp: int = 1) -> np.ndarray:
    """The local lattice vector (ghosts included) of a global lattice vector. Images of the
    split axis' periodicity take their masters' values: a slab cannot give the two cells that
    share a seam node different values there. The serial loop, like the reference, keeps an
    image's own initial value until the first solve distributes the constraints; the two agree
    whenever the initial condition is periodic along the split axis."""
    Ng = v.size // ncomp
    P = slab.plane_size
    out = np.empty(ncomp * slab.n_nodes)
    planes = np.array([slab.global_plane(L) for L in range(slab.local_planes)])
    for c in range(ncomp):
        g = v[c * Ng:(c + 1) * Ng].reshape(-1, P)
        out[c * slab.n_nodes:(c + 1) * slab.n_nodes] = g[planes].ravel()
    return out


# ---------------------------------------------------------------------------------------------
# local solvers: the GPU engine of one rank, or (for tests) the oracle
# ---------------------------------------------------------------------------------------------
class EngineLocal:
    """The GPU engine on one rank's slab; its work is queued on torch's current stream so the
    exchange (torch tensors) and the engine order themselves without host synchronisation."""

    device = "cuda"

    def __init__(self, problem):
        import torch
        self.p = problem
        self.torch = torch
        # torch's default stream is the legacy stream (handle 0); the engine takes it as
        # cudaStreamLegacy (1) because a null stream selects the handle's own stream
        problem.lib.ppf_set_stream(problem.h, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream or 1))

    def vector(self, f: int):
        return self.p.device_view(f, 0)

    def commit(self, f: int, v):  # views write through
        pass

    def increment_block(self, b: int, is_output: bool):
        self.p.increment_block(b, is_output)

    def end_increment(self) -> bool:
        """True when the increment produced a non-finite value."""
        from . import capi
        try:
            self.p.end_increment()
        except capi.PPFError as e:
            if e.code == capi.PPF_ERR_NAN:
                return True
            raise
        return False

    def get(self, f: int, age: int) -> np.ndarray:
        return self.p.download(f, age=age)

    def zeros(self, n: int):
        return self.torch.zeros(n, dtype=self.torch.float64, device="cuda")

    def apply(self, b: int, which: int, src, scale: int):
        """S op(src) of block b on device vectors (which 0: compute_rhs, 1: compute_lhs with
        src read through the homogeneous constraints); rows this rank owns are complete."""
        n = sum(self.p.field_length(f) for f in self.p.blocks[b].field_indices)
        dst = self.torch.empty(n, dtype=self.torch.float64, device="cuda")
        sp = ctypes.c_void_p(src.data_ptr()) if src is not None else None
        self.p._check(self.p.lib.ppf_apply_device(self.p.h, b, which, sp, ctypes.c_void_p(dst.data_ptr()), scale))
        return dst

    def set_current(self, f: int, v):
        self.p.device_view(f, 0).copy_(v)
        self.p.apply_constraints(f)

    def lhs_diagonal(self, b: int, tolerance_type: int):
        """The block's LHS diagonal on this slab (scaled by invM^1/2 unless AbsoluteResidual,
        zero entries one); rows this rank owns are complete."""
        self.p.set_linear_params(b, tolerance_type=tolerance_type)
        return self.torch.from_numpy(self.p.lhs_diagonal(b)).to("cuda")

    def constrained(self, f: int) -> np.ndarray:
        """Rows of field f the slab's constraint map ties to a master or a Dirichlet value."""
        m = self.p.constraint_map(f).astype(np.int64)
        return m != np.arange(m.size)



# ---------------------------------------------------------------------------------------------
# halo exchange and the increment loop
# ---------------------------------------------------------------------------------------------
class HaloExchange:
    """Moves ghost node planes between neighbours with torch.distributed point-to-point
    messages (or a local copy when a rank is its own neighbour)."""

    def __init__(self, slab: Slab, dist=None):
        self.slab = slab
        self.dist = dist

    def _ranges(self, planes: tuple[int, int], ncomp: int):
        P, N = self.slab.plane_size, self.slab.n_nodes
        return [(c * N + planes[0] * P, c * N + planes[1] * P) for c in range(ncomp)]

    def exchange(self, v, ncomp: int):
        """Fills the ghost planes of the local lattice vector v (torch tensor) in place. Each
        component's plane range is one contiguous slice of v, so it is sent from and received
        into a view of v directly: no packing or unpacking copies."""
        s = self.slab
        send_l = self._ranges(s.send_left_planes(), ncomp) if s.left is not None else []
        send_r = self._ranges(s.send_right_planes(), ncomp) if s.right is not None else []
        recv_r = self._ranges(s.recv_right_planes(), ncomp) if s.right is not None else []
        recv_l = self._ranges(s.recv_left_planes(), ncomp) if s.left is not None else []
        if s.size == 1:
            # the rank is its own neighbour (periodic split axis): local copies (the ranges of a
            # pair never overlap: the sent planes are owned, the received ones ghosts)
            for (a, b), (c, d) in zip(send_l, recv_r):
                v[c:d].copy_(v[a:b])
            for (a, b), (c, d) in zip(send_r, recv_l):
                v[c:d].copy_(v[a:b])
            return
        # With two periodic ranks both neighbours are the same process: messages carry a
        # direction and component tag (gloo), and every rank posts in the same order (leftward
        # sends, rightward sends, receipts of leftward messages, of rightward messages) so that
        # backends that pair point-to-point messages by order (NCCL) match them too.
        LEFTWARD, RIGHTWARD = 1, 2
        reqs = []
        for c, (a, b) in enumerate(send_l):
            reqs.append(self.dist.isend(v[a:b], s.left, tag=8 * LEFTWARD + c))
        for c, (a, b) in enumerate(send_r):
            reqs.append(self.dist.isend(v[a:b], s.right, tag=8 * RIGHTWARD + c))
        for c, (a, b) in enumerate(recv_r):
            reqs.append(self.dist.irecv(v[a:b], s.right, tag=8 * LEFTWARD + c))
        for c, (a, b) in enumerate(recv_l):
            reqs.append(self.dist.irecv(v[a:b], s.left, tag=8 * RIGHTWARD + c))
        for r in reqs:
            r.wait()


class ShardedExplicit:
    """The explicit increment loop of one simulation over all ranks: after every block that ran,
    the ghost planes of its fields are refreshed from the neighbours."""

    def __init__(self, slab: Slab, local, fields, blocks, dist=None):
        for b in blocks:
            if b.solve_type not in (Explicit, Constant):
                raise ValueError("the sharded loop runs explicit, constant and post-processing blocks")
        self.slab, self.local, self.fields, self.blocks = slab, local, fields, blocks
        self.halo = HaloExchange(slab, dist)
        self.dist = dist
        self.increment = 0

    def _ncomp(self, f: int) -> int:
        return 1 if self.fields[f].field_type == 0 else self.slab.mesh.dim

    def refresh(self, f: int):
        v = self.local.vector(f)
        self.halo.exchange(v, self._ncomp(f))
        self.local.commit(f, v)

    def run(self, n_increments: int, output_every: int = 0):
        while self.increment <= n_increments:
            inc = self.increment
            is_output = output_every > 0 and inc % output_every == 0
            for b, blk in enumerate(self.blocks):
                due = blk.solve_timing not in (PostProcess, NucleationRate) or is_output
                # at increment 0 a Primary block keeps the initial condition, images included
                due = due and not (inc == 0 and blk.solve_timing == Primary)
                self.local.increment_block(b, is_output)
                if due:
                    for f in blk.field_indices:
                        self.refresh(f)
            bad = self.local.end_increment()
            if self.dist is not None and self.slab.size > 1:
                torch = __import__("torch")
                flag = torch.tensor([1 if bad else 0], dtype=torch.int32, device=self.local.device)
                self.dist.all_reduce(flag, op=self.dist.ReduceOp.MAX)
                bad = bool(flag.item())
            if bad:
                raise FloatingPointError(f"non-finite value at increment {inc}")
            self.increment += 1

    def owned(self, f: int, age: int) -> np.ndarray:
        """This rank's owned planes of field f (all components, component-major)."""
        return owned_part(self.slab, self.local.get(f, age), self._ncomp(f))


def owned_part(slab: Slab, v: np.ndarray, ncomp: int) -> np.ndarray:
    """The owned planes of a local lattice vector (all components, component-major)."""
    n, P = slab.n_nodes, slab.plane_size
    lo, hi = slab.owned_planes()
    return np.concatenate([v[c * n + lo * P:c * n + hi * P] for c in range(ncomp)])


def assemble(slabs: list[Slab], parts: list[np.ndarray], mesh: RectangularMesh, ncomp: int = 1) -> np.ndarray:
    """The global lattice vector from every rank's owned planes (periodic images of the split
    axis take their master's values, as distributed constraints leave them)."""
    nn = mesh.nodes
    P = slabs[0].plane_size
    nplanes = nn[-1]
    out = np.empty(ncomp * nplanes * P)
    for s, part in zip(slabs, parts):
        lo, hi = s.owned_planes()
        cnt = (hi - lo) * P
        g0 = s.global_plane(lo)
        for c in range(ncomp):
            out[c * nplanes * P + g0 * P:c * nplanes * P + g0 * P + cnt] = part[c * cnt:(c + 1) * cnt]
    if slabs[0].periodic:
        for c in range(ncomp):
            base = c * nplanes * P
            out[base + (nplanes - 1) * P:base + nplanes * P] = out[base:base + P]
    return out


def local_workload(wl, slab: Slab):
    """A copy of a workload restricted to a rank's slab (mesh and initial condition). A face of
    the split axis next to a ghost cell layer is interior to the global mesh: Dirichlet
    conditions on its boundary id are dropped there (boundary ids 2 axis and 2 axis + 1)."""
    w = copy.copy(wl)
    w.mesh = slab.mesh
    w.initial = {f: local_from_global(slab, v, 1 if wl.fields[f].field_type == 0 else wl.mesh.dim)
                 for f, v in wl.initial.items()}
    interior = set()
    if slab.left is not None:
        interior.add(2 * slab.axis)
    if slab.right is not None:
        interior.add(2 * slab.axis + 1)
    fields = []
    for fa in wl.fields:
        fa = copy.copy(fa)
        fa.dirichlet = {key: v for key, v in fa.dirichlet.items() if key[1] not in interior}
        fields.append(fa)
    w.fields = fields
    return w


def _tridiag_max(a, b) -> float:
    """Largest eigenvalue of the symmetric tridiagonal matrix (diagonal a, off-diagonal b) by
    Sturm-count bisection inside its Gershgorin interval."""
    m = len(a)
    if not m:
        return 1.0
    lo, hi = a[0], a[0]
    for i in range(m):
        r = (abs(b[i - 1]) if i > 0 else 0.0) + (abs(b[i]) if i + 1 < m else 0.0)
        lo, hi = min(lo, a[i] - r), max(hi, a[i] + r)

    def below(x):
        cnt, q = 0, a[0] - x
        if q < 0:
            cnt += 1
        for i in range(1, m):
            qq = 1e-300 if q == 0.0 else q
            q = a[i] - x - b[i - 1] * b[i - 1] / qq
            if q < 0:
                cnt += 1
        return cnt

    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if below(mid) >= m:
            hi = mid
        else:
            lo = mid
        if hi - lo <= 1e-14 * max(1.0, abs(hi)):
            break
    return hi


class ShardedLinear:
    """The CG solve of a single-field Linear block over all ranks: deal.II's SolverCG as
    LinearSolver::solve_impl / do_linear_solve run it (linear_solver.h:305-402), with no
    preconditioner or a Chebyshev one, from the previous solution of the block (zero at first), to
    ||S (b - A x)|| < tolerance x normalization (S = invM^1/2 unless AbsoluteResidual;
    linear_solver.h:414-427). Vectors are local lattice vectors (ghost planes included); each
    operator apply first refreshes the ghost planes of its input; inner products sum the owned
    rows and are all-reduced. The solution becomes the field's current vector (constraints
    distributed, ghost planes refreshed)."""

    def __init__(self, slab: Slab, local, fields, blocks, global_mesh: RectangularMesh, dist=None):
        self.slab, self.local, self.fields, self.blocks, self.dist = slab, local, fields, blocks, dist
        self.halo = HaloExchange(slab, dist)
        self.volume = float(np.prod([global_mesh.size[d] for d in range(global_mesh.dim)]))
        self.x = {}
        self.eig = {}
        self.iterations = {}
        self.residual = {}

    def _ncomp(self, f: int) -> int:
        return 1 if self.fields[f].field_type == 0 else self.slab.mesh.dim

    def _owned(self, ncomp: int):
        n, P = self.slab.n_nodes, self.slab.plane_size
        lo, hi = self.slab.owned_planes()
        return [(c * n + lo * P, c * n + hi * P) for c in range(ncomp)]

    def _global_index(self, ncomp: int) -> np.ndarray:
        """Global lattice index (component-major) of every local row."""
        sl = self.slab
        P, n = sl.plane_size, sl.n_nodes
        N_global = sl.plane_size * (sl.degree * sl.n_cells + 1)
        planes = np.array([sl.global_plane(L) for L in range(sl.local_planes)], dtype=np.int64)
        node = (planes[:, None] * P + np.arange(P, dtype=np.int64)[None, :]).ravel()
        return np.concatenate([c * N_global + node for c in range(ncomp)])

    def _estimate_eig(self, b, A, inv_diag, f, ncomp, owned, eig_its, smoothing_range):
        """Largest eigenvalue of D^-1 A from eig_its CG steps on A x = pattern, x0 = 0, pattern
        the global lattice index mod 11 minus its mean over the unconstrained rows (the engine's
        and the oracle's estimate), reduced over the ranks; lambda_max x 1.2 and
        lambda_min = lambda_max / range as the Chebyshev interval."""
        torch = __import__("torch")
        cons = self.local.constrained(f)
        gi = self._global_index(ncomp)
        own = np.zeros(gi.size, dtype=bool)
        for a, e in owned:
            own[a:e] = True
        pat = (gi % 11).astype(np.float64)
        free = own & ~cons
        sums = torch.tensor([pat[free].sum(), float(free.sum())], dtype=torch.float64, device=inv_diag.device)
        if self.dist is not None and self.slab.size > 1:
            self.dist.all_reduce(sums, op=self.dist.ReduceOp.SUM)
        mean = float(sums[0]) / max(1.0, float(sums[1]))
        rhs = torch.from_numpy(np.where(cons, 0.0, pat - mean)).to(inv_diag.device)
        x = torch.zeros_like(rhs)
        r = rhs.clone()
        z = inv_diag * r
        p = z.clone()
        rz, r0 = self.dot(r, z, owned), self.dot(r, r, owned)
        al, be = [], []
        for _ in range(eig_its):
            q = A(p)
            pq = self.dot(p, q, owned)
            if pq <= 0.0 or not np.isfinite(pq):
                break
            alpha = rz / pq
            x += alpha * p
            r -= alpha * q
            al.append(alpha)
            if np.sqrt(self.dot(r, r, owned)) < 1e-10 * np.sqrt(r0):
                break
            z = inv_diag * r
            rzn = self.dot(r, z, owned)
            beta = rzn / rz
            rz = rzn
            be.append(beta)
            p = z + beta * p
        m = len(al)
        a = [1.0 / al[i] + (be[i - 1] / al[i - 1] if i > 0 else 0.0) for i in range(m)]
        o = [np.sqrt(max(0.0, be[i])) / al[i] for i in range(m - 1)]
        lmax = 1.2 * _tridiag_max(a, o)
        return lmax, lmax / smoothing_range

    def dot(self, u, v, owned) -> float:
        torch = __import__("torch")
        s = torch.zeros(1, dtype=torch.float64, device=u.device)
        for a, b in owned:
            s += torch.dot(u[a:b], v[a:b])
        if self.dist is not None and self.slab.size > 1:
            self.dist.all_reduce(s, op=self.dist.ReduceOp.SUM)
        return float(s.item())

    def solve(self, b: int, tolerance_type: int = 0, tolerance: float = 1e-10, max_iterations: int = 1000,
              preconditioner: int = 0, smoother_degree: int = 5, smoothing_range: float = 15.0,
              eig_cg_iterations: int = 10):
        """preconditioner 0: none; 1: Chebyshev (PreconditionerType::Chebyshev) of
        smoother_degree steps on the inverse diagonal, the interval from eig_cg_iterations
        CG-Lanczos steps (estimated at the block's first solve, the diagonal at every solve)."""
        blk = self.blocks[b]
        if len(blk.field_indices) != 1:
            raise ValueError("the sharded linear solve covers single-field Linear blocks")
        f = blk.field_indices[0]
        if any(v != 0.0 for v in self.fields[f].dirichlet.values()):
            raise NotImplementedError("the sharded linear solve takes homogeneous Dirichlet values")
        ncomp = self._ncomp(f)
        owned = self._owned(ncomp)
        scale = 0 if tolerance_type == 0 else 2
        norm = 1.0
        if tolerance_type in (1, 3):
            norm *= np.sqrt(self.volume)
        tol = tolerance * norm  # one field: sqrt(n_fields) = 1 (tolerance types 1 and 2)

        def A(v):
            self.halo.exchange(v, ncomp)
            return self.local.apply(b, 1, v, scale)

        rhs = self.local.apply(b, 0, None, scale)
        if preconditioner == 1:
            inv_diag = 1.0 / self.local.lhs_diagonal(b, tolerance_type)
            if b not in self.eig:
                self.eig[b] = self._estimate_eig(b, A, inv_diag, f, ncomp, owned, eig_cg_iterations, smoothing_range)
            lmax, lmin = self.eig[b]
            theta, delta = 0.5 * (lmax + lmin), 0.5 * (lmax - lmin)
            sigma = theta / delta

            def M(rr):  # Chebyshev of the first kind from a zero start (the oracle's smoother)
                xx = self.local.zeros(rr.numel())
                u = self.local.zeros(rr.numel())
                rho_prev = 1.0 / sigma
                for k in range(smoother_degree):
                    res_k = rr if k == 0 else rr - A(xx)
                    if k == 0:
                        c1, c2 = 0.0, 1.0 / theta
                    else:
                        rho = 1.0 / (2.0 * sigma - rho_prev)
                        c1, c2 = rho * rho_prev, 2.0 * rho / delta
                        rho_prev = rho
                    u = c1 * u + c2 * inv_diag * res_k
                    xx = xx + u
                return xx
        elif preconditioner == 0:
            def M(rr):
                return rr
        else:
            raise ValueError("the sharded linear solve takes no preconditioner (0) or Chebyshev (1)")
        x = self.x.get(b)
        if x is None:
            x = self.local.zeros(rhs.numel())
        r = rhs - A(x)
        res = np.sqrt(self.dot(r, r, owned))
        it = 0
        if res >= tol:
            z = M(r)
            p = z.clone()
            rz = self.dot(r, z, owned)
            while it < max_iterations:
                q = A(p)
                alpha = rz / self.dot(p, q, owned)
                x += alpha * p
                r -= alpha * q
                it += 1
                res = np.sqrt(self.dot(r, r, owned))
                if res < tol:
                    break
                z = M(r)
                rzn = self.dot(r, z, owned)
                beta = rzn / rz
                rz = rzn
                p = z + beta * p
        self.x[b] = x
        self.iterations[b], self.residual[b] = it, res / norm
        self.halo.exchange(x, ncomp)
        self.local.set_current(f, x)
        return it, res / norm

    def owned(self, f: int) -> np.ndarray:
        """This rank's owned planes of field f's current vector."""
        return owned_part(self.slab, self.local.get(f, 0), self._ncomp(f))
