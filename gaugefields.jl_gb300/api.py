"""Host-side mirror of the Gaugefields.jl interface for the SU(3) hot path.

Names follow the reference (Julia `f!` becomes Python `f_`); every call goes
through the C-ABI of libgfgb300.so, so the CUDA kernels do all the arithmetic.
Reference citations are paths inside Gaugefields.jl.

Host arrays use the reference's layouts (see include/gaugefields_gb300.h):
  links   : complex128 array (4, V, 3, 3) indexed [mu, lex, j, i]
            (the column-major (3,3,NX,NY,NZ,NT) array of each direction)
  momenta : float64 array (4, V, 8) indexed [mu, lex, a]
"""
import atexit
import ctypes
import math
import os
from collections import namedtuple

import numpy as np

from . import _lib
from ._lib import MDParams, call

__all__ = [
    "GB300Backend", "gauge_configuration", "measure_plaquette", "calculate_Plaquette", "construct_staple_",
    "calculate_Polyakov_loop", "measure_polyakov_loop",
    "gauge_momenta", "gaussian_momenta_", "gaussian_momenta", "GaugeAction", "push_", "evaluate_GaugeAction",
    "QPQ", "PQP", "OmelyanPQP", "md_driver", "md_step_size", "md_hamiltonian", "md_potential", "md_force_",
    "md_action_workspace", "update_gaugefields_", "update_momenta_", "md_step_", "md_trajectory_",
    "hmc_update_", "STOUT_Layer", "CovNeuralnet", "stout_smearing", "smear", "calc_smearedU", "back_prop",
    "get_parameter_derivatives",
    "Gradientflow", "gradient_flow", "flow_", "add_force_", "energy_density_plaquette", "substitute_U_",
    "similar", "clear_U_", "normalize_U_", "copy_configuration_", "copy_configuration", "save_configuration", "load_configuration_", "Oneinstanton_SUN_embedded",
    "MDActionSet", "MDForceGroup", "SextonWeingarten", "rectangle_sum", "Gradientflow_general",
]


_SHUTDOWN = [False]


@atexit.register
def _mark_shutdown():
    # At interpreter exit the objects below are finalised in no particular
    # order; the process is ending, so device memory is left to the driver.
    _SHUTDOWN[0] = True


def _live():
    return not _SHUTDOWN[0] and _lib._lib is not None


class GB300Backend:
    """Backend selector for gauge_configuration (cf. LatticeMatricesBackend,
    src/API.jl:6-27): one GB300, even/odd SoA storage, no halo, no MPI."""

    def __init__(self, device=0):
        self.device = int(device)


class _Context:
    """Owns one gf_ctx (lattice geometry + stream + reduction scratch)."""

    def __init__(self, L, device=0):
        lib = _lib.load()
        arr = (ctypes.c_int * 4)(*[int(x) for x in L])
        h = ctypes.c_void_p()
        rc = lib.gf_ctx_create(arr, int(device), ctypes.byref(h))
        _lib.check(rc, None)
        self.h = h
        self.L = tuple(int(x) for x in L)
        self.V = int(np.prod(self.L))
        self.device = device

    def sync(self):
        call("gf_ctx_synchronize", self.h, ctx=self.h)

    def set_stream(self, stream_handle):
        call("gf_ctx_set_stream", self.h, ctypes.c_void_p(stream_handle), ctx=self.h)

    def __del__(self):
        try:
            if getattr(self, "h", None) and _live():
                _lib._lib.gf_ctx_destroy(self.h)
                self.h = None
        except Exception:
            pass


class _Field:
    def __init__(self, ctx, kind):
        self.ctx = ctx
        self.kind = kind
        h = ctypes.c_void_p()
        call("gf_field_alloc", ctx.h, int(kind), ctypes.byref(h), ctx=ctx.h)
        self.h = h

    def device_ptr(self):
        p = ctypes.c_void_p()
        call("gf_field_device_ptr", self.h, ctypes.byref(p))
        return p.value

    def nbytes(self):
        n = ctypes.c_size_t()
        call("gf_field_bytes", self.h, ctypes.byref(n))
        return n.value

    def __del__(self):
        try:
            if getattr(self, "h", None) and _live():
                _lib._lib.gf_field_free(self.h)
                self.h = None
        except Exception:
            pass


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


class Gaugefields4D:
    """U: the four SU(3) link directions of a 4D lattice on the GPU
    (Gaugefields_4D_MPILattice, src/4D/mpi_jacc/gaugefields_4D_MPILattice.jl:34-121).
    kind GF_LINK64 (complex128) or GF_MAT64 for general matrices."""

    NC = 3
    Dim = 4

    def __init__(self, ctx, kind=_lib.GF_LINK64):
        self.ctx = ctx
        self.field = _Field(ctx, kind)

    @property
    def L(self):
        return self.ctx.L

    @property
    def NV(self):
        return self.ctx.V

    def __len__(self):
        return 4

    def similar(self):
        return Gaugefields4D(self.ctx, self.field.kind)

    def to_host(self):
        out = np.empty((4, self.NV, 3, 3), dtype=np.complex128)
        call("gf_download_links", self.ctx.h, self.field.h, _ptr(out), ctx=self.ctx.h)
        return out

    def from_host(self, arr):
        arr = np.ascontiguousarray(arr, dtype=np.complex128)
        if arr.size != 36 * self.NV:
            raise ValueError("link array has %d elements; expected %d" % (arr.size, 36 * self.NV))
        call("gf_upload_links", self.ctx.h, self.field.h, _ptr(arr), ctx=self.ctx.h)
        return self


class TAGaugefields4D:
    """Conjugate momenta / forces: 8 su(3) coefficients per link
    (TA_Gaugefields_4D_MPILattice, src/4D/mpi_jacc/TA_gaugefields_4D_MPILattice.jl:4-72)."""

    NumofBasis = 8

    def __init__(self, ctx):
        self.ctx = ctx
        self.field = _Field(ctx, _lib.GF_MOM64)

    def __len__(self):
        return 4

    def similar(self):
        return TAGaugefields4D(self.ctx)

    def to_host(self):
        out = np.empty((4, self.ctx.V, 8), dtype=np.float64)
        call("gf_download_mom", self.ctx.h, self.field.h, _ptr(out), ctx=self.ctx.h)
        return out

    def from_host(self, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        if arr.size != 32 * self.ctx.V:
            raise ValueError("momentum array has %d elements; expected %d" % (arr.size, 32 * self.ctx.V))
        call("gf_upload_mom", self.ctx.h, self.field.h, _ptr(arr), ctx=self.ctx.h)
        return self

    def __mul__(self, other):
        """P*P = sum_a p_a^2 (TA_gaugefields_4D_serial.jl:106-129). Only the
        self product (the kinetic term) is provided on the device."""
        if other is not self:
            raise NotImplementedError("only P*P (the kinetic term) is provided")
        out = ctypes.c_double()
        call("gf_kinetic", self.ctx.h, self.field.h, ctypes.byref(out), ctx=self.ctx.h)
        return out.value


# ---------------------------------------------------------------------------
# configurations and measurements (src/API.jl)
# ---------------------------------------------------------------------------
def gauge_configuration(lattice, backend=None, colors=3, halo=1, start="cold", seed=None, eltype=np.complex128,
                        verbose=0):
    """gauge_configuration(L; start=:cold|:hot, seed) (src/API.jl:178-251).

    The hot start is Haar-random SU(3) per link (Philox4x32-10 keyed by seed)."""
    backend = backend or GB300Backend()
    if not isinstance(backend, GB300Backend):
        raise ValueError("this package provides the GB300Backend only")
    L = tuple(int(x) for x in lattice)
    if len(L) != 4:
        raise ValueError("the GB300 backend is 4D; got %d dimensions" % len(L))
    if any(x <= 0 for x in L):
        raise ValueError("lattice extents must be positive; got %s" % (L,))
    if colors != 3:
        raise ValueError("the GB300 backend implements SU(3) only; got colors=%d" % colors)
    if halo < 0:
        raise ValueError("halo must be nonnegative; got %d" % halo)
    if start not in ("cold", "hot"):
        raise ValueError("start must be :cold or :hot; got %s" % start)
    if np.dtype(eltype) != np.complex128:
        raise ValueError("gauge_configuration stores complex128 links; use md_driver(precision='mixed') for fp32")
    ctx = _Context(L, backend.device)
    U = Gaugefields4D(ctx)
    if start == "cold":
        call("gf_cold_start", ctx.h, U.field.h, ctx=ctx.h)
    else:
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        call("gf_hot_start", ctx.h, U.field.h, ctypes.c_uint64(int(seed)), ctx=ctx.h)
    return U


def Oneinstanton_SUN_embedded(NC, NX, NY, NZ, NT, NDW=0, center=None, radius=None, sign=1, block=(1, 2),
                              backend=None):
    """Oneinstanton_SUN_embedded(NC, NX, NY, NZ, NT; center, radius, sign, block)
    (src/AbstractGaugefields.jl:1495-1581): the lattice SU(2) instanton placed
    in the colour rows and columns `block` of SU(3) links. The links are built
    on the host (special.py) and uploaded, as the reference builds them on the
    host before copying them to its lattice (its default centre L/2 + 1/2 and
    radius NX div 2)."""
    from . import special
    if NC != 3:
        raise ValueError("the GB300 backend implements SU(3) only; got NC=%d" % NC)
    if not isinstance(NDW, (int, np.integer)) or NDW < 0:
        raise ValueError("NDW must be a nonnegative integer; got %r" % (NDW,))
    L = (NX, NY, NZ, NT)
    links = special.oneinstanton_sun_embedded(NC, L, center=center, radius=radius, sign=sign, block=block)
    U = gauge_configuration(L, backend=backend, start="cold")
    return U.from_host(links)


# ---------------------------------------------------------------------------
# configuration files (src/API.jl:711-826)
# ---------------------------------------------------------------------------
def save_configuration(filename, U, format="ildg", precision="field", append=False):
    """save_configuration(filename, U; format=:ildg|:bridge, precision) (src/API.jl:711-726).

    The links are downloaded in the reference layout and written as one LIME
    message (format "ildg", ildg.py) or as Bridge++ text (format "bridge",
    bridge.py). For ILDG, precision "field" writes the fields' own 64 bits; 32
    or 64 choose the stored reals; append=True adds the configuration after
    the ones already in the file. Portable JLD2 output is not built."""
    if format == "bridge":
        if precision != "field" or append:
            raise ValueError("Bridge output does not accept format keywords")
        from . import bridge
        bridge.write(filename, U.to_host(), U.L)
        return None
    if format != "ildg":
        raise ValueError("format must be :ildg or :bridge for the GB300 backend (JLD2 output is not built); got %s"
                         % format)
    if precision == "field":
        precision = 64
    if precision not in (32, 64):
        raise ValueError("ILDG precision must be :field, 32, or 64; got %r" % (precision,))
    from . import ildg
    ildg.write(filename, U.to_host(), U.L, precision, append=append)
    return None


def load_configuration_(U, filename, format="ildg", index=1):
    """load_configuration!(U, filename; format=:ildg|:bridge) (src/API.jl:784-826):
    for ILDG the configuration `index` of the file (1 = the first, as the
    reference loads) into U, whose lattice must match the file's."""
    if format == "bridge":
        from . import bridge
        U.from_host(bridge.read(filename, U.L))
        return U
    if format != "ildg":
        raise ValueError("format must be :ildg or :bridge for the GB300 backend (JLD2 input is not built); got %s"
                         % format)
    from . import ildg
    links, _ = ildg.read(filename, L=U.L, index=index)
    U.from_host(links)
    return U


def similar(U):
    return U.similar()


def substitute_U_(A, B):
    """substitute_U!(A, B): A <- B (src/4D/mpi_jacc/gaugefields_4D_MPILattice.jl:509)."""
    call("gf_field_copy", A.ctx.h, A.field.h, B.field.h, ctx=A.ctx.h)


def copy_configuration_(destination, source):
    """copy_configuration!(destination, source) (src/API.jl:300-322): a
    complete configuration into compatible storage, returned. Different
    numbers of directions or lattice sizes raise (the reference's
    DimensionMismatch, a ValueError here)."""
    if len(destination) != len(source):
        raise ValueError("destination and source have different numbers of directions")
    if tuple(destination.L) != tuple(source.L):
        raise ValueError("destination and source lattice sizes differ")
    if destination.ctx is not source.ctx:
        destination.from_host(source.to_host())
    else:
        substitute_U_(destination, source)
    return destination


def copy_configuration(source):
    """copy_configuration(source) (src/API.jl:324-328): an independent copy."""
    return copy_configuration_(similar(source), source)


def clear_U_(A):
    call("gf_field_zero", A.ctx.h, A.field.h, ctx=A.ctx.h)


def normalize_U_(U):
    """normalize_U!(U) (src/AbstractGaugefields.jl:3378-3457, normalize3! per
    link): Gram-Schmidt of rows 1-2, row 3 the conjugate cross product, in
    fp64 on the device."""
    if U.field.kind != _lib.GF_LINK64:
        raise ValueError("normalize_U_ needs an fp64 link field")
    call("gf_reunitarize", U.ctx.h, U.field.h, ctx=U.ctx.h)


def calculate_Plaquette(U, temp=None, staple=None):
    """Sum over mu of Re tr(U_mu V_mu^dag)/2 (src/AbstractGaugefields.jl:2684-2699)."""
    out = ctypes.c_double()
    call("gf_plaquette", U.ctx.h, U.field.h, ctypes.byref(out), ctx=U.ctx.h)
    return out.value


def calculate_Polyakov_loop(U, temp1=None, temp2=None):
    """calculate_Polyakov_loop(U, temp1, temp2) (src/AbstractGaugefields.jl:
    2929-2956): the mean over the first time slice of tr of the product of
    the time links, a complex number; deterministic."""
    out = (ctypes.c_double * 2)()
    call("gf_polyakov_loop", U.ctx.h, U.field.h, out, ctx=U.ctx.h)
    return complex(out[0], out[1])


def measure_polyakov_loop(U, normalize=True):
    """measure_polyakov_loop(U; normalize=true) (src/API.jl:412-417)."""
    v = calculate_Polyakov_loop(U)
    return v / U.NC if normalize else v


def measure_plaquette(U, normalize=True):
    """measure_plaquette (src/API.jl:395-404): divided by 6*V*NC by default."""
    value = calculate_Plaquette(U)
    if not normalize:
        return value
    return value / (6 * U.NV * 3)


def energy_density_plaquette(U):
    """Plaquette-defined E = 2 sum_{mu<nu} Re tr(1 - P_munu) per site = 36 (1 - <P>)."""
    return 36.0 * (1.0 - measure_plaquette(U))


def construct_staple_(V, U, mu, temp=None):
    """construct_staple!(V, U, mu) (src/AbstractGaugefields.jl:2873-2923), mu 1-based
    as in the reference; the staple is written into direction slot mu of V."""
    if not 1 <= mu <= 4:
        raise ValueError("mu must be in 1..4")
    call("gf_staple", U.ctx.h, U.field.h, int(mu) - 1, V.field.h, ctx=U.ctx.h)
    return V


def gauge_momenta(U):
    """Zero-valued momenta compatible with U (src/API.jl:333)."""
    P = TAGaugefields4D(U.ctx)
    call("gf_field_zero", U.ctx.h, P.field.h, ctx=U.ctx.h)
    return P


def gaussian_momenta_(momenta, sigma=1.0, seed=None, sweep=0):
    """gaussian_momenta!(P; seed, sweep, sigma) (src/API.jl:341-368): p_a ~
    N(0, sigma^2), the unit-variance draws of (seed, sweep) scaled by sigma."""
    if sweep < 0:
        raise ValueError("sweep must be nonnegative; got %d" % sweep)
    if not math.isfinite(sigma):
        raise ValueError("sigma must be finite; got %s" % (sigma,))
    if seed is None:
        seed = int.from_bytes(os.urandom(8), "little")
    P = momenta
    call("gf_gaussian_momenta", P.ctx.h, P.field.h, ctypes.c_uint64(int(seed)), ctypes.c_uint64(int(sweep)),
         ctx=P.ctx.h)
    if sigma != 1.0:
        call("gf_mom_scale", P.ctx.h, P.field.h, ctypes.c_double(sigma), ctx=P.ctx.h)
    return P


def gaussian_momenta(U, sigma=1.0, seed=None, sweep=0):
    return gaussian_momenta_(gauge_momenta(U), sigma=sigma, seed=seed, sweep=sweep)


# ---------------------------------------------------------------------------
# gauge action (src/action/GaugeActions.jl)
# ---------------------------------------------------------------------------
_LOOPS = {"plaquette": "plaquette", ("plaquette", "plaquette_dag"): "plaquette",
          "rectangular": "rectangular", ("rectangular", "rectangular_dag"): "rectangular"}


class GaugeAction:
    """Wilson-loop action (src/action/GaugeActions.jl). The GB300 backend
    implements the plaquette loops push!(action, beta/2, plaq U plaq^dag)
    (docs/src/hmc.md:146-150) and the rectangle loops push!(action, c,
    rect U rect^dag) of make_loops_fromname("rectangular") (e.g. Iwasaki or
    Symanzik improvement, docs/src/legacyapi.md:80-92)."""

    def __init__(self, U, hascovnet=False):
        self.terms = []
        self.hascovnet = hascovnet

    @property
    def beta(self):
        """Twice the plaquette coefficient (the Wilson beta)."""
        return 2.0 * sum(c for c, kind in self.terms if kind == "plaquette")

    @property
    def c_rect(self):
        """The rectangle coefficient (0 without rectangle loops)."""
        return sum(c for c, kind in self.terms if kind == "rectangular")


def push_(action_or_net, coefficient, loops=None):
    """push!(action, coefficient, loops) / push!(network, layer)."""
    if isinstance(action_or_net, CovNeuralnet):
        action_or_net.layers.append(coefficient)
        return action_or_net
    kind = _LOOPS.get(loops if not isinstance(loops, list) else tuple(loops))
    if kind is None:
        raise ValueError("the GB300 backend supports the plaquette and rectangular loops (with their conjugates); "
                         "got %r" % (loops,))
    c = float(coefficient.real) if isinstance(coefficient, complex) else float(coefficient)
    action_or_net.terms.append((c, kind))
    return action_or_net


def rectangle_sum(U):
    """sum_x sum_{mu<nu} Re tr of the two rectangles (1x2 and 2x1) of the
    plane at x: the loops of make_rect (src/autostaples/wilsonloops.jl:304-330)."""
    out = ctypes.c_double()
    call("gf_rectangle", U.ctx.h, U.field.h, ctypes.byref(out), ctx=U.ctx.h)
    return out.value


def evaluate_GaugeAction(action, U):
    """Traced lattice sum of the action's loops (GaugeActions.jl:132-142):
    beta/2 * sum tr(plaq + plaq^dag) = beta * sum Re tr P, plus
    c_rect * sum tr(rect + rect^dag) = 2 c_rect * sum Re tr R."""
    v = action.beta * calculate_Plaquette(U)
    if action.c_rect != 0.0:
        v += 2.0 * action.c_rect * rectangle_sum(U)
    return v


# ---------------------------------------------------------------------------
# MD driver (src/molecular_dynamics.jl)
# ---------------------------------------------------------------------------
class QPQ:
    """Leapfrog with half link steps at both ends (molecular_dynamics.jl:611-616)."""


class PQP:
    """Leapfrog with half momentum steps at both ends (molecular_dynamics.jl:604-609)."""


class OmelyanPQP:
    """Second-order minimum-norm integrator, the reference's custom-integrator
    example (docs/src/hmc.md:250-270): P(l e) Q(e/2) P((1-2l) e) Q(e/2) P(l e)."""

    def __init__(self, lam=0.1931833275037836):
        if not math.isfinite(lam):
            raise ValueError("lambda must be finite")
        self.lam = float(lam)


class MDActionSet:
    """MDActionSet(; name=action, ...) (molecular_dynamics.jl:45-66): named
    action providers whose potentials and forces add. On this backend the
    members are GaugeActions of plaquette and rectangle loops on the driver's
    (smeared) links. Their forces are linear in
    the loop coefficients, so the force of any group of members is the force
    of one action with the group's summed coefficients: a group's momentum
    update is one fused force pass."""

    def __init__(self, terms=None, **named):
        terms = dict(terms or {}, **named)
        if not terms:
            raise ValueError("an MDActionSet must contain at least one action provider")
        for name, a in terms.items():
            if not isinstance(a, GaugeAction) or not a.terms:
                raise ValueError("md_action_workspace is not implemented for %s (member %s)"
                                 % (type(a).__name__, name))
        self.terms = terms

    @property
    def beta(self):
        return sum(a.beta for a in self.terms.values())

    @property
    def c_rect(self):
        return sum(a.c_rect for a in self.terms.values())

    def _members(self, group):
        unknown = [n for n in group.names if n not in self.terms]
        if unknown:
            raise ValueError("the force group selects unknown actions %s; available names are %s"
                             % (tuple(unknown), tuple(self.terms)))
        return [self.terms[n] for n in group.names]

    def group_beta(self, group):
        return sum(a.beta for a in self._members(group))

    def group_c_rect(self, group):
        return sum(a.c_rect for a in self._members(group))


class MDForceGroup:
    """MDForceGroup(names...) (molecular_dynamics.jl:68-93): the members of an
    MDActionSet that one momentum update applies."""

    def __init__(self, *names):
        if len(names) == 1 and isinstance(names[0], (tuple, list)):
            names = tuple(names[0])
        if not names:
            raise ValueError("an MDForceGroup must contain at least one action name")
        if len(set(names)) != len(names):
            raise ValueError("an MDForceGroup must not contain duplicate action names: %s" % (names,))
        self.names = tuple(str(n) for n in names)


def _force_group(group):
    if isinstance(group, MDForceGroup):
        return group
    if isinstance(group, str):
        return MDForceGroup(group)
    if isinstance(group, (tuple, list)):
        return MDForceGroup(*group)
    raise ValueError("a force group is an action name, a tuple of names or an MDForceGroup; got %r" % (group,))


class SextonWeingarten:
    """SextonWeingarten(; slow, fast, n_fast, ordering=QPQ())
    (molecular_dynamics.jl:296-360): two force time scales. QPQ ordering: a
    half-duration fast evolution of n_fast QPQ substeps on each side of one
    full slow kick; PQP ordering: half slow kicks around one full-duration
    fast evolution (molecular_dynamics.jl:618-686). The steps run from the
    host through update_momenta_ and update_gaugefields_."""

    def __init__(self, *, slow, fast, n_fast, ordering=None):
        ordering = QPQ() if ordering is None else ordering
        if isinstance(n_fast, bool) or int(n_fast) != n_fast or n_fast <= 0:
            raise ValueError("n_fast must be positive; got %s" % (n_fast,))
        if not isinstance(ordering, (QPQ, PQP)):
            raise ValueError("SextonWeingarten ordering must be PQP() or QPQ(); got %s" % type(ordering).__name__)
        self.slow = _force_group(slow)
        self.fast = _force_group(fast)
        self.n_fast = int(n_fast)
        self.ordering = ordering


def _validate_integrator(integrator, action):
    """_validate_md_integrator (molecular_dynamics.jl:364-402)."""
    if not isinstance(integrator, SextonWeingarten):
        return
    if not isinstance(action, MDActionSet):
        raise ValueError("SextonWeingarten requires an MDActionSet; got %s" % type(action).__name__)
    slow, fast = integrator.slow.names, integrator.fast.names
    overlap = [n for n in slow if n in fast]
    if overlap:
        raise ValueError("slow and fast force groups overlap: %s" % (tuple(overlap),))
    unknown = [n for n in slow + fast if n not in action.terms]
    if unknown:
        raise ValueError("SextonWeingarten selects unknown actions %s; available names are %s"
                         % (tuple(unknown), tuple(action.terms)))
    omitted = [n for n in action.terms if n not in slow + fast]
    if omitted:
        raise ValueError("SextonWeingarten does not schedule actions %s" % (tuple(omitted),))


_PRECISION = {"fp64": _lib.GF_FP64, "mixed": _lib.GF_MIXED, "dfloat": _lib.GF_DFLOAT}


class MDDriver:
    def __init__(self, action, integrator, trajectory_length, steps, smearing, precision, reunitarize,
                 recompute=False):
        self.action = action
        self.integrator = integrator
        self.trajectory_length = trajectory_length
        self.steps = steps
        self.smearing = smearing
        self.precision = precision
        self.reunitarize = reunitarize
        self.recompute = recompute

    def params(self, group=None):
        """The gf_md_params of this driver; with a force group, beta is the
        group's summed coupling."""
        p = MDParams()
        if group is None:
            p.beta = self.action.beta
            p.c_rect = self.action.c_rect
        else:
            if not isinstance(self.action, MDActionSet):
                raise ValueError("a force group selects members of an MDActionSet; the driver holds a %s"
                                 % type(self.action).__name__)
            group = _force_group(group)
            p.beta = self.action.group_beta(group)
            p.c_rect = self.action.group_c_rect(group)
        p.tau = self.trajectory_length
        p.steps = self.steps
        if isinstance(self.integrator, OmelyanPQP):
            p.integrator = _lib.GF_OMELYAN
            p.lam = self.integrator.lam
        else:
            p.integrator = _lib.GF_PQP if isinstance(self.integrator, PQP) else _lib.GF_QPQ
        p.precision = _PRECISION[self.precision]
        rho = self.smearing.rhos() if self.smearing is not None else []
        p.nstout = len(rho)
        for i, r in enumerate(rho):
            p.rho[i] = r
        p.reunitarize = 1 if self.reunitarize else 0
        p.stout_recompute = 1 if self.recompute else 0
        return p


def md_driver(U, action, steps, trajectory_length=1.0, integrator=None, smearing=None, precision="fp64",
              reunitarize=True, recompute=False):
    """md_driver(U, action; steps, trajectory_length, integrator) (molecular_dynamics.jl:440-483).

    smearing: a CovNeuralnet of stout layers; the action is then evaluated on
    the smeared links and the force is back-propagated to the thin links.
    precision: "fp64" (plain form), "mixed" (fp32 force and stout on 12-real
    links; fp64-class Hamiltonian, Delta H, link updates and re-unitarisation)
    or "dfloat" (force, stout and link updates in double-float arithmetic on
    the fp32 pipes, fp64 links; fp64 Hamiltonian).
    recompute: the stout adjoint rebuilds each level's staple sum C instead of
    keeping it from the forward pass (less device memory).
    An integrator without an md_step! (neither a builtin, a SextonWeingarten
    nor a callable) is accepted here and rejected when a step runs, as in the
    reference (test/md_driver.jl:309-320)."""
    integrator = integrator if integrator is not None else QPQ()
    if len(U) != 4:
        raise ValueError("the gauge configuration has length %d; expected 4" % len(U))
    if steps <= 0:
        raise ValueError("steps must be positive; got %d" % steps)
    if not math.isfinite(trajectory_length):
        raise ValueError("trajectory_length must be finite; got %s" % trajectory_length)
    if trajectory_length == 0:
        raise ValueError("trajectory_length must not be zero")
    if precision not in _PRECISION:
        raise ValueError("precision must be 'fp64', 'mixed' or 'dfloat'")
    if not (isinstance(action, MDActionSet) or (isinstance(action, GaugeAction) and action.terms)):
        raise ValueError("md_action_workspace is not implemented for %s" % type(action).__name__)
    _validate_integrator(integrator, action)
    return MDDriver(action, integrator, float(trajectory_length), int(steps), smearing, precision, reunitarize,
                    recompute)


def md_step_size(driver):
    return driver.trajectory_length / driver.steps


def md_action_workspace(action, U):
    return None


def md_potential(action, U, workspace=None, smearing=None):
    """-Re(evaluate_GaugeAction)/NC (molecular_dynamics.jl:247)."""
    if smearing is not None:
        U = smear(U, smearing)
    out = ctypes.c_double()
    if action.c_rect != 0.0:
        call("gf_action_loops", U.ctx.h, U.field.h, ctypes.c_double(0.5 * action.beta), ctypes.c_double(action.c_rect),
             ctypes.byref(out), ctx=U.ctx.h)
    else:
        call("gf_action", U.ctx.h, U.field.h, ctypes.c_double(action.beta), ctypes.byref(out), ctx=U.ctx.h)
    return out.value


def md_force_(force, action, U, workspace=None, group=None):
    """md_force!(F, ::GaugeAction, U, ws) (molecular_dynamics.jl:251-267); for
    an MDActionSet the sum of its members' forces, or of a group's
    (molecular_dynamics.jl:200-236)."""
    if group is not None:
        if not isinstance(action, MDActionSet):
            raise ValueError("a force group selects members of an MDActionSet; got %s" % type(action).__name__)
        group = _force_group(group)
        beta, c_rect = action.group_beta(group), action.group_c_rect(group)
    else:
        beta, c_rect = action.beta, action.c_rect
    if c_rect != 0.0:
        call("gf_force_loops", U.ctx.h, U.field.h, ctypes.c_double(0.5 * beta), ctypes.c_double(c_rect),
             force.field.h, ctx=U.ctx.h)
    else:
        call("gf_force", U.ctx.h, U.field.h, ctypes.c_double(beta), force.field.h, ctx=U.ctx.h)
    return None


def md_hamiltonian(U, P, driver):
    """Potential (on smeared links if the driver smears) + P*P/2, fp64."""
    p = driver.params()
    out = ctypes.c_double()
    call("gf_hamiltonian", U.ctx.h, U.field.h, P.field.h, ctypes.byref(p), ctypes.byref(out), ctx=U.ctx.h)
    return out.value


def update_gaugefields_(U, P, step_size, driver):
    """U_mu <- exp(step_size P_mu) U_mu (molecular_dynamics.jl:513-531), in the
    driver's precision (double-float for the mixed and double-float forms)."""
    if not math.isfinite(step_size):
        raise ValueError("the gauge-field step size must be finite; got %s" % step_size)
    p = driver.params()
    call("gf_md_link_update", U.ctx.h, U.field.h, P.field.h, ctypes.c_double(step_size), ctypes.byref(p),
         ctx=U.ctx.h)
    return U


def update_momenta_(P, U, step_size, driver, group=None):
    """P <- P + step_size * F(U) (molecular_dynamics.jl:539-551) with the
    driver's action, smearing and precision; with a force group, only the
    selected members of the driver's MDActionSet (molecular_dynamics.jl:553-584)."""
    if not math.isfinite(step_size):
        raise ValueError("the momentum step size must be finite; got %s" % step_size)
    p = driver.params(group)
    call("gf_md_mom_update", U.ctx.h, P.field.h, U.field.h, ctypes.c_double(step_size), ctypes.byref(p),
         ctx=U.ctx.h)
    return P


def md_step_(integrator, U, P, step_size, driver):
    """One MD step (molecular_dynamics.jl:593-616). Custom integrators are
    callables f(U, P, step_size, driver) built from update_momenta_ and
    update_gaugefields_, as in the reference."""
    if isinstance(integrator, PQP):
        update_momenta_(P, U, step_size / 2, driver)
        update_gaugefields_(U, P, step_size, driver)
        update_momenta_(P, U, step_size / 2, driver)
    elif isinstance(integrator, OmelyanPQP):
        lam = integrator.lam
        update_momenta_(P, U, lam * step_size, driver)
        update_gaugefields_(U, P, 0.5 * step_size, driver)
        update_momenta_(P, U, (1 - 2 * lam) * step_size, driver)
        update_gaugefields_(U, P, 0.5 * step_size, driver)
        update_momenta_(P, U, lam * step_size, driver)
    elif isinstance(integrator, QPQ):
        update_gaugefields_(U, P, step_size / 2, driver)
        update_momenta_(P, U, step_size, driver)
        update_gaugefields_(U, P, step_size / 2, driver)
    elif isinstance(integrator, SextonWeingarten):
        _sexton_weingarten_step(integrator, U, P, step_size, driver)
    elif callable(integrator):
        integrator(U, P, step_size, driver)
    else:
        raise ValueError("md_step! is not implemented for %s" % type(integrator).__name__)


def _fast_evolution(U, P, duration, n, driver, fast):
    """n QPQ substeps of the fast group over `duration`, the half link steps
    between substeps applied as one (_md_fast_qpq!, molecular_dynamics.jl:618-633)."""
    h = duration / n
    update_gaugefields_(U, P, h / 2, driver)
    for i in range(n):
        update_momenta_(P, U, h, driver, fast)
        update_gaugefields_(U, P, h if i < n - 1 else h / 2, driver)


def _sexton_weingarten_step(sw, U, P, step_size, driver):
    """One Sexton-Weingarten step (molecular_dynamics.jl:635-686)."""
    if isinstance(sw.ordering, QPQ):
        _fast_evolution(U, P, step_size / 2, sw.n_fast, driver, sw.fast)
        update_momenta_(P, U, step_size, driver, sw.slow)
        _fast_evolution(U, P, step_size / 2, sw.n_fast, driver, sw.fast)
    else:
        update_momenta_(P, U, step_size / 2, driver, sw.slow)
        _fast_evolution(U, P, step_size, sw.n_fast, driver, sw.fast)
        update_momenta_(P, U, step_size / 2, driver, sw.slow)


MDResult = namedtuple("MDResult", ["initial_hamiltonian", "final_hamiltonian", "delta_hamiltonian"])


def md_trajectory_(U, P, driver, diagnostics=True):
    """md_trajectory!(U, P, driver) (molecular_dynamics.jl:712-730). The builtin
    QPQ/PQP/Omelyan run as one native call; SextonWeingarten and custom
    integrators step from the host through update_momenta_ and
    update_gaugefields_."""
    if isinstance(driver.integrator, (QPQ, PQP, OmelyanPQP)):
        p = driver.params()
        out = (ctypes.c_double * 3)()
        call("gf_md_trajectory", U.ctx.h, U.field.h, P.field.h, ctypes.byref(p), out, ctx=U.ctx.h)
        return MDResult(out[0], out[1], out[2]) if diagnostics else None
    h0 = md_hamiltonian(U, P, driver) if diagnostics else None
    eps = md_step_size(driver)
    for _ in range(driver.steps):
        md_step_(driver.integrator, U, P, eps, driver)
    if not diagnostics:
        return None
    h1 = md_hamiltonian(U, P, driver)
    return MDResult(h0, h1, h1 - h0)


HMCResult = namedtuple("HMCResult", ["initial_hamiltonian", "final_hamiltonian", "delta_hamiltonian", "accepted"])


def hmc_update_(U, P, driver, seed, sweep, unif):
    """Momentum refresh + md_trajectory! + Metropolis (docs/src/hmc.md:22-81):
    accept when Delta H <= 0 or unif < exp(-Delta H); a rejected trajectory
    restores U, and a non-finite Delta H restores U and raises. The builtin
    integrators run as one native call (gf_hmc_update); SextonWeingarten and
    custom integrators take the same steps from the host (a device copy of
    the links, gaussian_momenta_, md_trajectory_, the same test)."""
    if not 0.0 <= unif < 1.0:
        raise ValueError("unif must be in [0,1); got %s" % (unif,))
    if not isinstance(driver.integrator, (QPQ, PQP, OmelyanPQP)):
        backup = U.similar()
        substitute_U_(backup, U)
        gaussian_momenta_(P, seed=seed, sweep=sweep)
        res = md_trajectory_(U, P, driver)
        dh = res.delta_hamiltonian
        finite = math.isfinite(dh)
        accept = finite and (dh <= 0.0 or unif < math.exp(-dh))
        if not accept:
            substitute_U_(U, backup)
        if not finite:
            raise _lib.GFNonFinite(_lib.GF_ENAN, "hmc_update_: Delta H is not finite; configuration restored")
        return HMCResult(res.initial_hamiltonian, res.final_hamiltonian, dh, accept)
    p = driver.params()
    out = (ctypes.c_double * 4)()
    call("gf_hmc_update", U.ctx.h, U.field.h, P.field.h, ctypes.byref(p), ctypes.c_uint64(int(seed)),
         ctypes.c_uint64(int(sweep)), ctypes.c_double(unif), out, ctx=U.ctx.h)
    return HMCResult(out[0], out[1], out[2], bool(out[3]))


# ---------------------------------------------------------------------------
# stout smearing (src/smearing)
# ---------------------------------------------------------------------------
class STOUT_Layer:
    """Plaquette stout layer (stout_fast.jl:6-121): Ubar = exp(TA(C U^dag)) U."""

    def __init__(self, loops="plaquette", rho=0.1, U=None):
        names = [loops] if isinstance(loops, str) else list(loops)
        if names != ["plaquette"]:
            raise ValueError("the GB300 backend implements plaquette stout layers only")
        rhos = [rho] if np.isscalar(rho) else list(rho)
        if len(rhos) != 1:
            raise ValueError("rho must be a scalar or have one entry per loop")
        self.rho = float(rhos[0])


class CovNeuralnet:
    """Stack of smearing layers (Abstractsmearing.jl:61-99)."""

    def __init__(self, U=None):
        self.layers = []

    def rhos(self):
        return [l.rho for l in self.layers]

    def __len__(self):
        return len(self.layers)


def stout_smearing(U, loops="plaquette", rho=0.1):
    """stout_smearing(U; loops, rho) (src/API.jl:452-463): one plaquette layer."""
    net = CovNeuralnet(U)
    push_(net, STOUT_Layer(loops, rho, U))
    return net


class _StoutStack:
    """A gf_stout workspace (levels, stored C, back-propagation buffers)."""

    def __init__(self, ctx, rhos, precision="fp64", store=True):
        if not 1 <= len(rhos) <= _lib.GF_MAX_STOUT:
            raise ValueError("1..%d stout levels are supported" % _lib.GF_MAX_STOUT)
        self.ctx = ctx
        arr = (ctypes.c_double * len(rhos))(*rhos)
        h = ctypes.c_void_p()
        prec = _PRECISION[precision]
        call("gf_stout_create", ctx.h, len(rhos), arr, prec, 1 if store else 0, ctypes.byref(h), ctx=ctx.h)
        self.h = h
        self.precision = precision

    def __del__(self):
        try:
            if getattr(self, "h", None) and _live():
                _lib._lib.gf_stout_destroy(self.h)
                self.h = None
        except Exception:
            pass


SmearingResult = namedtuple("SmearingResult", ["configuration", "history", "derivative"])


def calc_smearedU(U, smearing, calcdSdU=False, temps=None):
    """Forward through every layer (Abstractsmearing.jl:237-272); the history
    is the native stack that keeps each level for back_prop."""
    stack = _StoutStack(U.ctx, smearing.rhos(), "fp64")
    Uout = U.similar()
    call("gf_stout_forward", U.ctx.h, stack.h, U.field.h, Uout.field.h, ctx=U.ctx.h)
    return Uout, stack, None


def smear(U, smearing, record=False, calcdSdU=False, temps=None):
    """smear(U, smearing; record) (src/API.jl:472-480)."""
    configuration, history, derivative = calc_smearedU(U, smearing, calcdSdU=calcdSdU, temps=temps)
    return SmearingResult(configuration, history, derivative) if record else configuration


def back_prop(dSdUbar, smearing, history, U):
    """back_prop(δ, net, Uout_multi, U) (Abstractsmearing.jl:316-411): dS/dU on
    the thin links from dS/dUbar (both general 3x3 fields, fp64)."""
    out = Gaugefields4D(U.ctx, _lib.GF_MAT64)
    call("gf_stout_backward", U.ctx.h, history.h, dSdUbar.field.h, out.field.h, ctx=U.ctx.h)
    return out


def get_parameter_derivatives(dSdUbar, smearing, U, precision="fp64"):
    """get_parameter_derivatives(δL, net, Uout_multi, Uin) (Abstractsmearing.jl:
    416-436, with parameter_derivatives of each STOUT_Layer, stout_fast.jl:
    371-386): dS/drho of every layer of `smearing` on the thin links U, given
    dS/dUbar of the top level (a general 3x3 fp64 field). Returns a list with
    one value per layer."""
    rhos = smearing.rhos()
    stack = _StoutStack(U.ctx, rhos, precision)
    if precision == "mixed":
        d = Gaugefields4D(U.ctx, _lib.GF_MAT32)
        call("gf_field_copy", U.ctx.h, d.field.h, dSdUbar.field.h, ctx=U.ctx.h)
    else:
        d = dSdUbar
    out = (ctypes.c_double * len(rhos))()
    call("gf_stout_param_derivatives", U.ctx.h, stack.h, U.field.h, d.field.h, out, ctx=U.ctx.h)
    return list(out)


# ---------------------------------------------------------------------------
# gradient flow (src/smearing/gradientflow.jl)
# ---------------------------------------------------------------------------
class Gradientflow:
    """Wilson flow with the Luescher RK3 integrator (gradientflow.jl:118-161).
    precision: "fp64" (the reference's arithmetic) or "dfloat" (the force and
    the exponentials in double-float arithmetic on the fp32 pipes, fp64
    fields)."""

    def __init__(self, U, Nflow=1, eps=0.01, precision="fp64"):
        if precision not in ("fp64", "dfloat"):
            raise ValueError("the flow's precision must be 'fp64' or 'dfloat'")
        self.Nflow = int(Nflow)
        self.eps = float(eps)
        self.precision = precision


class Gradientflow_general:
    """Gradient flow of a general loop action (gradientflow.jl:42-118,
    240-336): Gradientflow_general(U, linknames, linkvalues; Nflow, eps) with
    the loop names "plaquette" and "rectangular" and real coefficients (each
    set with its conjugate loops); the force is TA(U dS/dU)."""

    def __init__(self, U, linknames, linkvalues, Nflow=1, eps=0.01):
        names = [linknames] if isinstance(linknames, str) else list(linknames)
        values = [linkvalues] if np.isscalar(linkvalues) else list(linkvalues)
        if len(names) != len(values):
            raise ValueError("one coefficient per loop name is needed; got %d names and %d values"
                             % (len(names), len(values)))
        self.c_plaq, self.c_rect = 0.0, 0.0
        for n, v in zip(names, values):
            if isinstance(v, complex) or not np.isreal(v):
                raise ValueError("the GB300 backend takes real loop coefficients; got %r" % (v,))
            if n == "plaquette":
                self.c_plaq += float(v)
            elif n == "rectangular":
                self.c_rect += float(v)
            else:
                raise ValueError("the GB300 backend supports the plaquette and rectangular loops; got %r" % (n,))
        self.Nflow = int(Nflow)
        self.eps = float(eps)


def gradient_flow(U, loops=None, coefficients=None, steps=1, step_size=0.01, precision="fp64"):
    """gradient_flow(U; steps, step_size) and gradient_flow(U, loops,
    coefficients; steps, step_size) (src/API.jl:420-438); precision "dfloat"
    selects the double-float Wilson flow (plaquette action only)."""
    if steps <= 0:
        raise ValueError("steps must be positive; got %d" % steps)
    if step_size <= 0:
        raise ValueError("step_size must be positive; got %s" % step_size)
    if loops is None and coefficients is None:
        return Gradientflow(U, Nflow=steps, eps=step_size, precision=precision)
    if loops is None or coefficients is None:
        raise ValueError("a general-action flow needs both loops and coefficients")
    if precision != "fp64":
        raise ValueError("the general-action flow runs in fp64")
    return Gradientflow_general(U, loops, coefficients, Nflow=steps, eps=step_size)


def flow_(U, g):
    """flow!(U, g) (gradientflow.jl:171-238; Gradientflow_general :240-336)."""
    if isinstance(g, Gradientflow_general):
        call("gf_flow_loops", U.ctx.h, U.field.h, ctypes.c_double(g.eps), int(g.Nflow), ctypes.c_double(g.c_plaq),
             ctypes.c_double(g.c_rect), ctx=U.ctx.h)
        return U
    call("gf_flow_precision", U.ctx.h, U.field.h, ctypes.c_double(g.eps), int(g.Nflow), _PRECISION[g.precision],
         ctx=U.ctx.h)
    return U


def add_force_(F, U, plaqonly=True, factor=1.0):
    """add_force!(F, U; plaqonly=true, factor) (AbstractGaugefields.jl:2717-2763)."""
    if not plaqonly:
        raise ValueError("only plaqonly=true is implemented (the general branch of the reference is unused)")
    call("gf_flow_force", U.ctx.h, U.field.h, F.field.h, ctypes.c_double(factor), ctx=U.ctx.h)
    return F
