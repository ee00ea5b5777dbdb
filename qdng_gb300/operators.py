"""Host-side mirror of the QDng operator tree on the propagation path.

The classes keep the reference's names and the meaning of their XML
attributes, and flatten the tree into the qdg_hplan_desc the C ABI takes:

* ``GridNablaSq(mass=[...], method, order, pbc)`` -- src/qdlib/OGridNablaSq.cpp:28-58, Diff.cpp:149-200
* ``GridGMat(dims, gmat, G, Gdef, coup)`` -- src/qdlib/OGridGMat.cpp:142-386 (G-matrix kinetic energy)
* ``GridHOFD(deriv, order, dim, pbc, mass)`` -- src/qdlib/OGridHOFD.cpp:32-128 (finite differences)
* ``GridPotential(values)``     -- src/qdlib/OGridPotential.cpp:26-109 (setzero/offset/scale)
* ``GridDipole(mu, laser)``     -- src/qdlib/OGridDipole.cpp:18-60, Laser.cpp:125-128
* ``GridNAC([f_0, ...], mass, sign)`` -- src/qdlib/OGridNAC.cpp:26-148 (first-derivative coupling)
* ``Sum([...])``                -- src/qdlib/OSum.cpp:28-72
* ``Multistate({(i, j): op})``  -- src/qdlib/OMultistate.cpp:100-241 (hermitian: (i,j) also acts at (j,i),
  unless ``nonhermitian`` or both (i,j) and (j,i) are given, OMultistate.cpp:52-53,83-85)
* ``DMultistate({(i, j): op})`` -- src/qdlib/ODMultistate.cpp:35-182 (GSPO members)

Errors follow the reference's exceptions: ``EParamProblem`` for bad
parameters, ``EIncompatible`` for operator/wave-function mismatches.
"""
import ctypes as C

import numpy as np

from . import abi


class EParamProblem(ValueError):
    """src/tools/Exception.h EParamProblem."""


class EIncompatible(TypeError):
    """src/tools/Exception.h EIncompatible."""


class EOverflow(ArithmeticError):
    """src/tools/Exception.h EOverflow."""


class EIOError(IOError):
    """src/tools/Exception.h EIOError."""


class GridSystem:
    """QDng GridSystem: dim 0 fastest, dx = (xmax - xmin)/(N - 1) (GridSystem.cpp:207-211)."""

    def __init__(self, n, xmin, xmax):
        n = [int(v) for v in np.atleast_1d(n)]
        xmin = [float(v) for v in np.atleast_1d(xmin)]
        xmax = [float(v) for v in np.atleast_1d(xmax)]
        if not (1 <= len(n) <= abi.QDG_MAX_DIMS) or len(xmin) != len(n) or len(xmax) != len(n):
            raise EParamProblem("invalid grid dimensions")
        for i in range(len(n)):
            if n[i] < 1:
                raise EParamProblem("Zero points grid defined")
            if xmax[i] - xmin[i] <= 0:
                raise EParamProblem("Zero length grid defined")
        self.n, self.xmin, self.xmax = n, xmin, xmax

    @property
    def ndims(self):
        return len(self.n)

    @property
    def npts(self):
        return int(np.prod(self.n))

    @property
    def dx(self):
        return [(self.xmax[i] - self.xmin[i]) / (self.n[i] - 1) for i in range(self.ndims)]

    def axes(self):
        """Coordinate axes, x_i = xmin + i*dx."""
        return [self.xmin[i] + np.arange(self.n[i]) * self.dx[i] for i in range(self.ndims)]

    def mesh(self):
        """Coordinate arrays shaped (n[D-1], ..., n[0]) -- C order with dim 0 fastest."""
        ax = self.axes()
        grids = np.meshgrid(*ax[::-1], indexing="ij")
        return grids[::-1]

    def to_c(self):
        g = abi.Grid()
        g.ndims = self.ndims
        for i in range(self.ndims):
            g.n[i] = self.n[i]
            g.xmin[i] = self.xmin[i]
            g.xmax[i] = self.xmax[i]
        return g

    def __eq__(self, other):
        return (isinstance(other, GridSystem) and self.n == other.n
                and np.allclose(self.xmin, other.xmin, rtol=0, atol=0)
                and np.allclose(self.xmax, other.xmax, rtol=0, atol=0))


class Operator:
    def terms(self, row, col, group, ctx):
        raise NotImplementedError


class GridNablaSq(Operator):
    """Kinetic energy -1/(2m) d^2/dx^2 per dimension, by FFT (``method="FFT"``)
    or by central finite differences of even ``order`` 2..50 (``method="HOFD"``,
    Diff.cpp:149-200, default order 8 = DIFF_DEF_ORDER, Diff.h:20) with
    ``pbc`` periodic boundaries (one-dimensional grids)."""

    def __init__(self, mass, method="FFT", order=8, pbc=False):
        mass = [float(m) for m in np.atleast_1d(mass)]
        if len(mass) < 1:
            raise EParamProblem("Nabla operator needs at least one dimension")
        for m in mass:
            if m == 0:
                raise EParamProblem("Zero mass defined")
            if m < 0:
                raise EIncompatible("negative masses (excluded dimensions) are not supported")
        self.mass = mass
        if method not in ("FFT", "HOFD"):
            raise EParamProblem("Unknown differenciation method", method)
        self.method = method
        self.order = int(order) if method == "HOFD" else 0
        self.pbc = bool(pbc) and method == "HOFD"
        if method == "HOFD" and (self.order > 50 or self.order % 2 != 0 or self.order < 2):
            # HOFD::_CheckSetup (HOFD.h:82-89)
            raise EParamProblem("Invalid order of FD derivative", self.order)

    def terms(self, row, col, group, ctx):
        if row != col:
            raise EIncompatible("GridNablaSq must sit on the diagonal")
        if len(self.mass) != ctx.grid.ndims:
            raise EIncompatible("OGridNablaSq: Number of dims doesn't match WF")
        if self.pbc and ctx.grid.ndims != 1:
            raise EIncompatible("HOFD with pbc on grids of more than one dimension")
        t = abi.HTerm()
        t.kind, t.row, t.col, t.grid, t.laser, t.group = abi.TERM_KINETIC, row, col, -1, -1, group
        for i, m in enumerate(self.mass):
            t.mass[i] = m
        t.fd_order = self.order
        t.flags = 1 if self.pbc else 0
        return [t]


class GridHOFD(Operator):
    """OGridHOFD (src/qdlib/OGridHOFD.cpp:32-128): central finite differences
    of even ``order`` (2..50) along each dimension (``dim`` = -1) or one
    dimension, first (``deriv=1``) or second (``deriv=2``) derivative, zero
    boundaries or periodic ones (``pbc``).  With ``mass`` the factor is
    -1/(2 m) of the last dimension's mass for every dimension (as the
    reference assigns it), else 1.  Defaults as the reference's: deriv 1,
    order 2, all dimensions."""

    def __init__(self, deriv=1, order=2, dim=-1, pbc=False, mass=None):
        self.deriv, self.order, self.dim, self.pbc = int(deriv), int(order), int(dim), bool(pbc)
        # HOFD::_CheckSetup (HOFD.h:82-89)
        if self.order > 50 or self.order % 2 != 0 or self.order < 2:
            raise EParamProblem("Invalid order of FD derivative", self.order)
        if self.deriv not in (1, 2):
            raise EParamProblem("Invalid FD derivative", self.deriv)
        self.mass = None if mass is None else [float(m) for m in np.atleast_1d(mass)]
        if self.mass is not None:
            if len(self.mass) < 1:
                raise EParamProblem("HOFD operator needs at least one mass defintion")
            if any(m == 0 for m in self.mass):
                raise EParamProblem("Zero mass defined")

    def terms(self, row, col, group, ctx):
        if row != col:
            raise EIncompatible("GridHOFD must sit on the diagonal")
        nd = ctx.grid.ndims
        if self.dim >= nd or self.dim < -1:
            raise EParamProblem("Invalid number of active dimension", self.dim)
        if self.mass is not None and len(self.mass) < nd:
            raise EIncompatible("GridHOFD: fewer masses than dimensions")
        t = abi.HTerm()
        t.kind, t.row, t.col, t.grid, t.laser, t.group = abi.TERM_HOFD, row, col, -1, self.dim, group
        t.fd_order = self.order
        t.flags = (1 if self.pbc else 0) | (2 if self.deriv == 1 else 0) | (4 if self.mass is not None else 0)
        if self.mass is not None:
            for i in range(nd):
                t.mass[i] = self.mass[i]
        return [t]


class GridGMat(Operator):
    """OGridGMat (src/qdlib/OGridGMat.cpp:142-248, 307-386): the G-matrix
    kinetic energy -1/2 sum_ij d/dx_j G_ij(x) d/dx_i with FFT derivatives.

    ``gmat`` maps (i, j), i >= j, to the grid array of G_ij (the files
    ``<gmat>_ij`` of the reference); ``G`` lists constant elements and
    ``Gdef`` the source of each element ('g' grid, 'c' constant, 'x' none),
    both in lower-triangle order (0,0), (1,0), (1,1), (2,0), ...
    (ReorderLowerTriangular, tools/helpers.h:95-112).  Without ``Gdef`` every
    element is a constant when ``G`` is given, else a grid.  ``coup=False``
    drops the off-diagonal elements.  The chain-rule form, PML and finite
    difference derivatives are not provided."""

    def __init__(self, dims, gmat=None, G=None, Gdef=None, coup=True, chainrule=False, pml=False,
                 method="FFT"):
        n = int(dims)
        if n < 1:
            raise EParamProblem("G-matrix operator needs at least one dimension")
        if chainrule or pml or method != "FFT":
            raise EIncompatible("GridGMat: only the FFT form without chain rule and PML is provided")
        self.n = n
        self.coup = bool(coup)
        nl = n * (n + 1) // 2
        src = ["c" if G is not None else "g"] * nl
        if Gdef is not None:
            for k, c in enumerate(list(Gdef)[:nl]):
                src[k] = c
        const = [0.0] * nl
        if G is not None:
            for k, v in enumerate(list(np.atleast_1d(G))[:nl]):
                const[k] = float(v)
        gmat = dict(gmat or {})
        self.elements = []  # per lower-triangle element: (source code, array or constant)
        for i in range(n):
            for j in range(i + 1):
                k = i * (i + 1) // 2 + j
                if i != j and not self.coup:
                    self.elements.append((0, None))
                elif src[k] == "g":
                    if (i, j) not in gmat:
                        raise EParamProblem("No G-matrix elements given")
                    self.elements.append((1, np.array(gmat[(i, j)], dtype=np.float64).reshape(-1)))
                elif src[k] == "c":
                    self.elements.append((2, const[k]))
                else:
                    self.elements.append((0, None))

    def terms(self, row, col, group, ctx):
        if row != col:
            raise EIncompatible("GridGMat must sit on the diagonal")
        if self.n != ctx.grid.ndims:
            raise EIncompatible("Gmatrix element is incompatible with wave function")
        t = abi.HTerm()
        t.kind, t.row, t.col, t.laser, t.group = abi.TERM_GMAT, row, col, -1, group
        flags = 0
        arrs = []
        for k, (code, val) in enumerate(self.elements):
            if code == 1:
                if val.size != ctx.grid.npts:
                    raise EIncompatible("Gmatrix element is incompatible with wave function")
                arrs.append(val)
            elif code == 2:
                arrs.append(np.full(ctx.grid.npts, val))
            else:
                arrs.append(np.zeros(ctx.grid.npts))
            flags |= code << (2 * k)
        t.grid = ctx.add_grids(arrs)
        t.flags = flags
        return [t]


class GridPotential(Operator):
    """V(x) psi. ``values`` has grid shape or npts entries (dim 0 fastest)."""

    def __init__(self, values, setzero=False, offset=0.0, scale=1.0):
        v = np.array(values, dtype=np.float64).reshape(-1)
        if setzero:
            v = v - v.min()
        if offset != 0:
            v = v + offset
        if scale != 1:
            v = v * scale
        self.values = v

    def terms(self, row, col, group, ctx):
        if self.values.size != ctx.grid.npts:
            raise EIncompatible("GridPotential parameters are not compatible with wave function")
        t = abi.HTerm()
        t.kind, t.row, t.col, t.laser, t.group = abi.TERM_POTENTIAL, row, col, -1, group
        t.grid = ctx.add_grid(self.values)
        return [t]


class GridDipole(Operator):
    """-mu(x) E(t) psi with E(step) = laser[step]."""

    def __init__(self, mu, laser):
        self.mu = np.array(mu, dtype=np.float64).reshape(-1)
        self.laser = np.array(laser, dtype=np.float64).reshape(-1)

    def terms(self, row, col, group, ctx):
        if self.mu.size != ctx.grid.npts:
            raise EIncompatible("GridDipole parameters are not compatible with wave function")
        t = abi.HTerm()
        t.kind, t.row, t.col, t.group = abi.TERM_DIPOLE, row, col, group
        t.grid = ctx.add_grid(self.mu)
        t.laser = ctx.add_laser(self.laser)
        return [t]


def _bw_lowpass(n, center, order):
    """FunctionGenerator::BwLowpass (src/math/math_functions.h:60-70): 1 / (1 + (i / center)^(2 order))."""
    i = np.arange(n, dtype=np.float64)
    with np.errstate(divide="ignore", over="ignore"):
        return 1.0 / (1.0 + np.power(i / center, 2.0 * order))


def _bw_highpass(n, center, order):
    """FunctionGenerator::BwHighpass (src/math/math_functions.h:40-50): 1 / (1 + (center / i)^(2 order))."""
    i = np.arange(n, dtype=np.float64)
    with np.errstate(divide="ignore", over="ignore"):
        return 1.0 / (1.0 + np.power(center / i, 2.0 * order))


class Gobbler(Operator):
    """OGobbler (src/qdlib/OGobbler.cpp): Butterworth filter functions along
    the dimensions.  ``lp`` / ``rp`` map a dimension to the cut-off x of a
    left pass (keeps smaller x) / right pass (keeps larger x); ``order`` the
    filter order (default 20); ``gain`` a factor.  With ``nip`` the filter is
    a negative imaginary potential, H psi += -i W psi, else H psi += W psi.
    Emax = gain, Emin = -i gain (nip) or 0 (OGobbler.cpp:161-170)."""

    def __init__(self, dims=None, lp=None, rp=None, order=20, gain=1.0, nip=False):
        if order < 1:
            raise EParamProblem("Filter order to small")
        self.dims = dims
        self.lp = dict(lp or {})
        self.rp = dict(rp or {})
        self.order = int(order)
        self.gain = float(gain)
        self.nip = bool(nip)
        self.W = None

    def filter(self, grid):
        """OGobbler::_Init (OGobbler.cpp:30-84) on the grid (dim 0 fastest)."""
        if self.dims is not None and self.dims != grid.ndims:
            raise EIncompatible("OGobbler: Number of dims doesn't match WF")
        shape = tuple(reversed(grid.n))
        f = np.zeros(shape) if self.nip else np.ones(shape)
        dx = grid.dx
        for d in range(grid.ndims):
            bshape = [1] * grid.ndims
            bshape[grid.ndims - 1 - d] = grid.n[d]
            for side, table in (("lp", self.lp), ("rp", self.rp)):
                if d not in table:
                    continue
                x = (table[d] - grid.xmin[d]) / dx[d]
                if int(x) > grid.n[d] or int(x) < 0:
                    raise EParamProblem("Center of filter edge out of the grid")
                if side == "lp":
                    f = f * _bw_lowpass(grid.n[d], x, self.order).reshape(bshape)
                elif self.nip:
                    f = f + _bw_highpass(grid.n[d], x, self.order).reshape(bshape)
                else:
                    f = f * _bw_highpass(grid.n[d], x, self.order).reshape(bshape)
        if self.gain != 1:
            f = f * self.gain
        return np.ascontiguousarray(f).reshape(-1)

    def terms(self, row, col, group, ctx):
        if row != col:
            raise EIncompatible("Gobbler off the diagonal")
        if self.W is None or self.W.size != ctx.grid.npts:
            self.W = self.filter(ctx.grid)
        t = abi.HTerm()
        t.kind, t.row, t.col, t.group = abi.TERM_GOBBLER, row, col, group
        t.grid = ctx.add_grid(self.W)
        t.laser = 1 if self.nip else 0
        t.mass[0] = self.gain
        return [t]


class GridNAC(Operator):
    """Non-adiabatic first-derivative coupling (OGridNAC::Apply,
    src/qdlib/OGridNAC.cpp:131-148):
    sign/(2 mass) * sum_d [f_d d/dx_d psi + d/dx_d (f_d psi)].
    ``nacme`` holds one coupling grid per dimension.  ``mass`` is used for
    one-dimensional grids only; with more dimensions the reference keeps
    mass = 1 and expects it folded into the coupling data (OGridNAC.cpp:83-85)."""

    def __init__(self, nacme, mass=None, sign=1.0):
        if isinstance(nacme, np.ndarray) and nacme.ndim == 1:
            nacme = [nacme]
        self.nacme = [np.array(f, dtype=np.float64).reshape(-1) for f in nacme]
        if len(self.nacme) < 1:
            raise EParamProblem("NAC got nonsense dims")
        self.mass = 1.0 if mass is None else float(mass)
        self.sign = float(sign)

    def terms(self, row, col, group, ctx):
        if len(self.nacme) != ctx.grid.ndims:
            raise EIncompatible("NAC: Psi has different num of dims")
        for f in self.nacme:
            if f.size != ctx.grid.npts:
                raise EIncompatible("GridNAC parameters are not compatible with wave function")
        t = abi.HTerm()
        t.kind, t.row, t.col, t.laser, t.group = abi.TERM_NAC, row, col, -1, group
        t.grid = ctx.add_grids(self.nacme)
        t.mass[0] = self.mass if ctx.grid.ndims == 1 else 1.0
        t.sign = self.sign
        return [t]


class Sum(Operator):
    def __init__(self, ops):
        if len(ops) == 0:
            raise EParamProblem("Sum Operator is empty")
        self.ops = list(ops)

    def terms(self, row, col, group, ctx):
        out = []
        for o in self.ops:
            out += o.terms(row, col, group, ctx)
        return out


class Multistate(Operator):
    """Operator matrix.  An element given at (i, j), i != j, also acts at
    (j, i), unless the matrix is non-hermitian: the ``nonhermitian``
    parameter, or elements given at both (i, j) and (j, i)."""

    def __init__(self, elements, nstates=None, nonhermitian=False):
        self.elements = dict(elements)
        n = 1 + max(max(i, j) for (i, j) in self.elements)
        self.nstates = nstates or n
        if self.nstates < 1:
            raise EParamProblem("Multistate operator is empty")
        both = any(i != j and (j, i) in self.elements for (i, j) in self.elements)
        self.nonhermitian = bool(nonhermitian) or both

    def terms(self, row, col, group, ctx):
        out = []
        for (i, j), o in sorted(self.elements.items()):
            out += o.terms(i, j, group, ctx)
        if self.nonhermitian:
            ctx.nonhermitian = True
        return out


class DMultistate(Multistate):
    """Multistate member of a GSPO split (diagonalisable per grid point or by FFT)."""


class _Ctx:
    def __init__(self, grid):
        self.grid = grid
        self.grids = []
        self.lasers = []
        self.nonhermitian = False

    def add_grid(self, v):
        for i, g in enumerate(self.grids):
            if g is v:
                return i
        self.grids.append(v)
        return len(self.grids) - 1

    def add_grids(self, vs):
        """Consecutive grid slots (a coupling grid per dimension); returns the first."""
        first = len(self.grids)
        self.grids.extend(vs)
        return first

    def add_laser(self, v):
        for i, g in enumerate(self.lasers):
            if g is v:
                return i
        self.lasers.append(v)
        return len(self.lasers) - 1


class HPlan:
    """A flattened Hamiltonian (qdg_hplan_desc) plus the arrays it points to."""

    def __init__(self, grid, hamiltonian=None, nstates=1, members=None):
        """hamiltonian: Sum/Multistate/single operator (Cheby, SIL, Arnoldi);
        members: [A, B, C, ...] GSPO split operators (OGSPO.cpp:71-85).
        Exactly one of them is given; a GSPO plan's H is the sum of its members."""
        self.grid = grid
        ctx = _Ctx(grid)
        terms = []
        if members is not None:
            for g, m in enumerate(members):
                if isinstance(m, Multistate):
                    nstates = max(nstates, m.nstates)
                terms += m.terms(0, 0, g, ctx)
        else:
            if isinstance(hamiltonian, Multistate):
                nstates = max(nstates, hamiltonian.nstates)
            terms += hamiltonian.terms(0, 0, 0, ctx)
        for t in terms:
            if t.row >= nstates or t.col >= nstates:
                raise EParamProblem("Multistate operator can only use WFs with same number of states")
        self.nstates = nstates
        self.terms = terms
        self.nonhermitian = ctx.nonhermitian
        npts = grid.npts
        self.grid_data = (np.concatenate(ctx.grids) if ctx.grids else np.zeros(1)).astype(np.float64)
        if ctx.lasers:
            nt = max(len(l) for l in ctx.lasers)
            lz = np.zeros((len(ctx.lasers), nt))
            for i, l in enumerate(ctx.lasers):
                lz[i, :len(l)] = l
            self.laser_data = lz.reshape(-1)
            self.laser_nt = nt
        else:
            self.laser_data = np.zeros(1)
            self.laser_nt = 0
        self.ngrids = len(ctx.grids)
        self._grids = list(ctx.grids)
        self.nlasers = len(ctx.lasers)
        self._terms_c = (abi.HTerm * max(1, len(terms)))(*terms)
        d = abi.HPlanDesc()
        d.grid = grid.to_c()
        d.nstates = nstates
        d.nterms = len(terms)
        d.terms = C.cast(self._terms_c, C.POINTER(abi.HTerm))
        d.ngrids = self.ngrids
        self._gd = np.ascontiguousarray(self.grid_data)
        d.grid_data = self._gd.ctypes.data_as(C.POINTER(C.c_double))
        d.nlasers = self.nlasers
        d.laser_nt = self.laser_nt
        self._ld = np.ascontiguousarray(self.laser_data)
        d.laser_data = self._ld.ctypes.data_as(C.POINTER(C.c_double))
        d.nonhermitian = 1 if self.nonhermitian else 0
        self.desc = d
        self.npts = npts

    @property
    def size(self):
        """Complex values of one wave function (all states)."""
        return self.npts * self.nstates

    def grid_of(self, op):
        """Index in grid_data of a GridPotential's values or a Gobbler's filter
        (the operator a filter's ref= names in QDng)."""
        v = op.W if isinstance(op, Gobbler) else getattr(op, "values", None)
        for i, g in enumerate(self._grids):
            if g is v:
                return i
        raise EParamProblem("operator not part of this Hamiltonian")
