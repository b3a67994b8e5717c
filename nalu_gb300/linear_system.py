"""Host-side mirror of the reference interfaces on the assembly path.

Names and argument meaning follow NaluCFD/Nalu so that a caller of
``LinearSystem`` / ``AssembleElemSolverAlgorithm`` / ``Kernel`` finds the same
surface; every call goes through the C ABI (``include/nalu_gb300.h``).

* ``LinearSystem``                 -- include/LinearSystem.h:39-167,
                                      src/TpetraLinearSystem.C
* ``AssembleElemSolverAlgorithm``  -- include/AssembleElemSolverAlgorithm.h:38-112
* ``*ElemKernel``                  -- include/kernel/Kernel.h:95-125 and the
                                      kernel sources named on each class
* ``AssembleFaceElemSolverAlgorithm`` -- src/AssembleFaceElemSolverAlgorithm.C,
                                      with the continuity inflow / open kernels

Kernels run as one fused device pass each (gather, master element, element
matrix, sumInto).  Several active kernels therefore add into the system one
after the other instead of into one shared element matrix; the sums are the
same up to floating-point summation order.
"""
from . import (FACE_CONTINUITY_INFLOW, FACE_CONTINUITY_OPEN, KERNEL_CONTINUITY_ADV, KERNEL_CONTINUITY_MASS,
               KERNEL_MOMENTUM_ADV_DIFF, KERNEL_MOMENTUM_MASS, KERNEL_MOMENTUM_UPW_ADV_DIFF, KERNEL_SCALAR_DIFF,
               default_assemble_opts, default_solver_opts)


class TimeIntegrator:
    """The TimeIntegrator values the kernels' setup() reads: time step and
    the BDF coefficients gamma1 phi^{n+1} + gamma2 phi^n + gamma3 phi^{n-1}
    (BDF1 by default)."""

    def __init__(self, dt=1.0, gamma1=1.0, gamma2=-1.0, gamma3=0.0):
        self.dt, self.gamma1, self.gamma2, self.gamma3 = dt, gamma1, gamma2, gamma3

    @staticmethod
    def of(ti):
        """accepts a TimeIntegrator, a (dt, gamma1[, gamma2, gamma3]) tuple or None"""
        if ti is None or isinstance(ti, TimeIntegrator):
            return ti
        return TimeIntegrator(*ti)


class Kernel:
    """Base of the element kernels (include/kernel/Kernel.h:95-125)."""

    kernel_id = None
    num_dof = 1

    def __init__(self, **opts):
        self.opts = default_assemble_opts(**opts)

    def setup(self, time_integrator=None):
        """Kernel::setup(const TimeIntegrator&)."""


class ScalarDiffElemKernel(Kernel):
    """src/kernel/ScalarDiffElemKernel.C: CVFEM diffusion of scalarQ with
    diffFluxCoeff (fields ``scalar_q`` and ``diff_coeff``)."""

    kernel_id = KERNEL_SCALAR_DIFF

    def __init__(self, shifted_grad_op=False):
        super().__init__(shifted_grad_op=int(shifted_grad_op))


class ContinuityAdvElemKernel(Kernel):
    """src/kernel/ContinuityAdvElemKernel.C: pressure-Poisson Laplacian and
    mass-flux residual (fields velocity, density, pressure, dpdx)."""

    kernel_id = KERNEL_CONTINUITY_ADV

    def __init__(self, shift_mdot=False, shift_poisson=False, reduced_sens=False):
        # SolutionOptions forces reduced sensitivities with the shifted Poisson
        # operator (src/SolutionOptions.C:719-724)
        reduced_sens = reduced_sens or shift_poisson
        super().__init__(shift_mdot=int(shift_mdot), shift_poisson=int(shift_poisson),
                         reduced_sens=int(reduced_sens))

    def setup(self, time_integrator=None):
        """projTimeScale = dt / gamma1 (ContinuityAdvElemKernel.C:79-84)."""
        ti = TimeIntegrator.of(time_integrator)
        if ti is not None:
            self.opts.proj_time_scale = ti.dt / ti.gamma1


class ContinuityMassElemKernel(Kernel):
    """src/kernel/ContinuityMassElemKernel.C: density time derivative at the
    sub-control volumes (fields density, density_n, density_nm1)."""

    kernel_id = KERNEL_CONTINUITY_MASS

    def __init__(self, lumped_mass=False):
        super().__init__(lumped_mass=int(lumped_mass))

    def setup(self, time_integrator=None):
        ti = TimeIntegrator.of(time_integrator) or TimeIntegrator()
        self.opts.dt, self.opts.gamma1, self.opts.gamma2, self.opts.gamma3 = ti.dt, ti.gamma1, ti.gamma2, ti.gamma3


class MomentumMassElemKernel(ContinuityMassElemKernel):
    """src/kernel/MomentumMassElemKernel.C: (rho u) time derivative and the
    Gjp source (fields density*, velocity, velocity_n, velocity_nm1, dpdx)."""

    kernel_id = KERNEL_MOMENTUM_MASS
    num_dof = 3

    def __init__(self, lumped_mass=False, balanced_force=False):
        Kernel.__init__(self, lumped_mass=int(lumped_mass), balanced_force=int(balanced_force))


class MomentumAdvDiffElemKernel(Kernel):
    """src/kernel/MomentumAdvDiffElemKernel.C: central advection with the SCS
    mass flow plus the full viscous stress (fields velocity, viscosity,
    mass_flow_rate_scs)."""

    kernel_id = KERNEL_MOMENTUM_ADV_DIFF
    num_dof = 3

    def __init__(self, include_divu=0.0, shifted_grad_op=False, skew_symmetric=False):
        super().__init__(include_divu=float(include_divu), shifted_grad_op=int(shifted_grad_op),
                         skew_symmetric=int(skew_symmetric))


class MomentumUpwAdvDiffElemKernel(Kernel):
    """src/kernel/MomentumUpwAdvDiffElemKernel.C: upwind/central blended
    advection (alpha, alpha_upw, upw_factor, classic Peclet blending with
    hybrid_factor, optional van Leer limiter) plus viscous stress."""

    kernel_id = KERNEL_MOMENTUM_UPW_ADV_DIFF
    num_dof = 3

    def __init__(self, alpha=0.0, alpha_upw=1.0, upw_factor=1.0, hybrid_factor=0.0, use_limiter=False,
                 include_divu=0.0, shifted_grad_op=False, skew_symmetric=False):
        super().__init__(alpha=float(alpha), alpha_upw=float(alpha_upw), upw_factor=float(upw_factor),
                         hybrid_factor=float(hybrid_factor), use_limiter=int(use_limiter),
                         include_divu=float(include_divu), shifted_grad_op=int(shifted_grad_op),
                         skew_symmetric=int(skew_symmetric))


class LinearSystem:
    """TpetraLinearSystem analogue on one GPU."""

    def __init__(self, ctx, num_dof=1):
        self.ctx = ctx
        self.numDof_ = num_dof
        self.linearSolveIterations_ = 0
        self.linearResidual_ = 0.0
        self.solver_opts = default_solver_opts()

    def buildElemToNodeGraph(self, parts=None):
        self.ctx.build_elem_graph(self.numDof_)

    def finalizeLinearSystem(self):
        """The graph, CRS arrays and slot tables are complete after buildElemToNodeGraph."""

    def zeroSystem(self):
        self.ctx.zero()

    def sumInto(self, elem_ids, lhs, rhs):
        self.ctx.sum_into(elem_ids, lhs, rhs)

    def applyDirichletBCs(self, nodes, bc_values, solution, beginPos=0, endPos=None):
        self.ctx.apply_dirichlet(nodes, bc_values, solution, beginPos, endPos)

    def resetRows(self, nodes, beginPos=0, endPos=None):
        self.ctx.reset_rows(nodes, beginPos, endPos)

    def loadComplete(self):
        self.ctx.load_complete()

    def solve(self, opts=None):
        info = self.ctx.solve(opts or self.solver_opts, raise_on_error=False)
        self.linearSolveIterations_ = info.iterations
        self.linearResidual_ = info.true_rel_res
        return info.status

    def graph(self):
        return self.ctx.graph()

    def values_and_rhs(self):
        return self.ctx.system()


class AssembleElemSolverAlgorithm:
    """Element loop driver (src/AssembleElemSolverAlgorithm.C:47-100)."""

    def __init__(self, linsys):
        self.linsys = linsys
        self.activeKernels_ = []

    def initialize_connectivity(self):
        self.linsys.buildElemToNodeGraph()

    def execute(self, time_integrator=None):
        for k in self.activeKernels_:
            if k.num_dof != self.linsys.numDof_:
                raise ValueError("kernel numDof does not match the linear system")
            k.setup(time_integrator)
            self.linsys.ctx.assemble(k.kernel_id, k.opts)


class ContinuityInflowElemKernel(Kernel):
    """src/kernel/ContinuityInflowElemKernel.C (field cont_velocity_bc)."""

    kernel_id = FACE_CONTINUITY_INFLOW

    def __init__(self, use_shifted=False):
        super().__init__(shift_mdot=int(use_shifted))

    def setup(self, time_integrator=None):
        ti = TimeIntegrator.of(time_integrator)
        if ti is not None:
            self.opts.proj_time_scale = ti.dt / ti.gamma1


class ContinuityOpenElemKernel(ContinuityInflowElemKernel):
    """src/kernel/ContinuityOpenElemKernel.C (fields pressure, pressure_bc,
    density, velocity, dpdx; the side set's dynamic pressure)."""

    kernel_id = FACE_CONTINUITY_OPEN

    def __init__(self, shift_mdot=False, shift_poisson=False, reduced_sens=False):
        Kernel.__init__(self, shift_mdot=int(shift_mdot), shift_poisson=int(shift_poisson),
                        reduced_sens=int(reduced_sens or shift_poisson))


class AssembleFaceElemSolverAlgorithm:
    """Face / face-element loop driver (src/AssembleFaceElemSolverAlgorithm.C)
    over one side set of the context (``Context.faceset_define`` or
    ``faceset_skin``)."""

    def __init__(self, linsys, side_set):
        self.linsys = linsys
        self.side_set = side_set
        self.activeKernels_ = []

    def execute(self, time_integrator=None):
        for k in self.activeKernels_:
            k.setup(time_integrator)
            self.linsys.ctx.assemble_faces(self.side_set, k.kernel_id, k.opts)
