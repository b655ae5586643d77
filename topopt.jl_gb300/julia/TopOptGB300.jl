"""
    TopOptGB300

Julia binding of libtopopt_gb300.so: a GB300 drop-in for TopOpt.jl's SIMP
compliance loop.  `FEASolver(GB300Solver, problem; xmin, penalty, ...)` returns
a solver whose `solver()` call, `ComplianceFun`, `VolumeFun`,
`DensityFilterFun` and `SensFilterFun` run on the GPU through `ccall`; the
design vector stays a plain `Vector{Float64}` on the host side of every call,
as in the reference.  Plug-in points used (TopOpt.jl paths):

  * `AbstractLinearSolver` (src/FEA/solvers_api.jl:44) -> `GB300Solver`
  * `FEASolver(::Type{S}, problem; kw...)` (solvers_api.jl:599-603) -> a
    `GB300FEASolver <: AbstractFEASolver` that never builds the E copies of Ke
    nor the sparse K (solvers_api.jl:492-494)
  * `ComplianceFun` call (src/Functions/compliance.jl:58-70); the generic rrule
    (compliance.jl:72-76) then returns `comp.grad`
  * `AbstractDensityFilter` / `AbstractSensFilter` subtypes with call + rrule
    (src/CheqFilters/CheqFilters.jl:34-41)

Indices cross the boundary 0-based (Julia dof d is d-1 in C).
"""
module TopOptGB300

using TopOpt
using TopOpt: PseudoDensities
using TopOpt.FEA: AbstractLinearSolver, AbstractFEASolver
using TopOpt.TopOptProblems: StiffnessTopOptProblem, getdh, getncells
using TopOpt.CheqFilters: AbstractDensityFilter, AbstractSensFilter
using TopOpt.Functions: ComplianceFun, VolumeFun
using TopOpt.Utilities: PowerPenaltyFun, getpenalty
using ChainRulesCore
using Ferrite
using SparseArrays

export GB300Solver, GB300FEASolver, GB300DensityFilter, GB300SensFilter, oc_update!, simp_step!
export BatchedSIMP, batch_step!, batch_results, WarmStartNet, attach_network!
export GB300FixedElementProjector, clear_fixed_elements!, GB300ProjectedDensityFilter, mma_update!, mma_reset!

const libtog = joinpath(@__DIR__, "..", "libtopopt_gb300.so")

const TOG_OK = Cint(0)
const TOG_NOT_CONVERGED = Cint(3)
const TOG_FP64 = Cint(0)
const TOG_FP32_IR = Cint(1)

struct GB300Solver <: AbstractLinearSolver end

struct ProblemDesc
    dim::Int32
    nel::NTuple{3,Int32}
    size::NTuple{3,Float64}
    E::Float64
    nu::Float64
    plane_stress::Int32
    xmin::Float64
    penalty::Float64
end

mutable struct SolveStats
    status::Int32
    iterations::Int32
    outer_iterations::Int32
    reserved::Int32
    rel_residual::Float64
    abs_residual::Float64
end
SolveStats() = SolveStats(0, 0, 0, 0, 0.0, 0.0)

last_error() = unsafe_string(ccall((:tog_last_error, libtog), Cstring, ()))

function check(code::Cint)
    code == TOG_OK && return nothing
    msg = last_error()
    code == Cint(1) && throw(ArgumentError(msg))
    code == TOG_NOT_CONVERGED && (@warn "GB300 PCG: $msg"; return nothing)  # cg! is silent at maxiter
    return error("libtopopt_gb300: $msg (status $code)")
end

mutable struct GB300FEASolver{T,TP<:StiffnessTopOptProblem} <: AbstractFEASolver
    problem::TP
    handle::Ptr{Cvoid}
    vars::Vector{T}
    u::Vector{T}
    penalty::PowerPenaltyFun{T}
    xmin::T
    cg_max_iter::Int
    abstol::T
    rtol::T
    precision::Cint
    warm_start::Bool
    stats::SolveStats
end

"""
    FEASolver(GB300Solver, problem; xmin=1e-3, penalty=PowerPenaltyFun(1.0),
              cg_max_iter=700, abstol=1e-7, rtol=sqrt(eps()), precision=:fp64,
              warm_start=false)

Same keywords and defaults as the reference's `FEASolver` (solvers_api.jl:468-489),
plus `rtol` (IterativeSolvers' reltol, exposed) and `precision` (`:fp64` or
`:fp32_ir`).  Inhomogeneous Dirichlet BCs are rejected as by CGMatrixFreeSolver.
"""
function TopOpt.FEA.FEASolver(::Type{GB300Solver}, problem::StiffnessTopOptProblem{dim,T};
                              xmin=T(1) / 1000, penalty=PowerPenaltyFun{T}(1), cg_max_iter=700,
                              abstol=T(1e-7), rtol=sqrt(eps(T)), precision=:fp64, warm_start=false,
                              conv=TopOpt.FEA.DefaultCriteria(), kwargs...) where {dim,T}
    ch = problem.ch
    any(!=(0), ch.inhomogeneities) && throw(ArgumentError(
        "GB300Solver supports homogeneous Dirichlet BCs only (as CGMatrixFreeSolver)"))
    rg = problem.rect_grid
    nel = ntuple(i -> i <= dim ? Int32(rg.nels[i]) : Int32(1), 3)
    sz = ntuple(i -> i <= dim ? Float64(rg.sizes[i]) : 1.0, 3)
    desc = Ref(ProblemDesc(Int32(dim), nel, sz, Float64(problem.E), Float64(problem.ν), Int32(0),
                           Float64(xmin), Float64(penalty.p)))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:tog_create, libtog), Cint, (Ref{ProblemDesc}, Ref{Ptr{Cvoid}}), desc, h))
    fixed = Int32.(ch.prescribed_dofs .- 1)
    check(ccall((:tog_set_fixed_dofs, libtog), Cint, (Ptr{Cvoid}, Int64, Ptr{Int32}), h[], length(fixed), fixed))
    f = Vector{Float64}(TopOpt.TopOptProblems.make_cload(problem))
    check(ccall((:tog_set_rhs, libtog), Cint, (Ptr{Cvoid}, Ptr{Float64}), h[], f))
    # conv (solvers_api.jl:482): EnergyCriteria runs as the FP64 solve's stop rule on the device
    check(ccall((:tog_set_convergence, libtog), Cint, (Ptr{Cvoid}, Int32), h[],
                conv isa TopOpt.FEA.EnergyCriteria ? Int32(1) : Int32(0)))
    nc = getncells(problem)
    prec = precision === :fp32_ir ? TOG_FP32_IR : TOG_FP64
    s = GB300FEASolver{T,typeof(problem)}(problem, h[], ones(T, nc), zeros(T, length(f)), penalty, T(xmin),
                                          cg_max_iter, T(abstol), T(rtol), prec, warm_start, SolveStats())
    finalizer(s) do x
        x.handle == C_NULL || ccall((:tog_destroy, libtog), Cint, (Ptr{Cvoid},), x.handle)
        x.handle = C_NULL
    end
    return s
end

TopOpt.Utilities.getpenalty(s::GB300FEASolver) = s.penalty
function TopOpt.Utilities.setpenalty!(s::GB300FEASolver, p)
    s.penalty = p isa PowerPenaltyFun ? p : PowerPenaltyFun(oftype(s.xmin, p))
    check(ccall((:tog_set_penalty, libtog), Cint, (Ptr{Cvoid}, Float64), s.handle, s.penalty.p))
    return s
end

"""`solver()`: solve K(vars) u = f on the GPU (replaces solvers_api.jl:285-374)."""
function (s::GB300FEASolver)(args...; kwargs...)
    length(s.vars) == getncells(s.problem) || throw(DimensionMismatch("vars"))
    check(ccall((:tog_set_vars, libtog), Cint, (Ptr{Cvoid}, Ptr{Float64}), s.handle, s.vars))
    check(ccall((:tog_solve, libtog), Cint,
                (Ptr{Cvoid}, Cint, Float64, Float64, Int32, Int32, Ref{SolveStats}),
                s.handle, s.precision, s.rtol, s.abstol, s.cg_max_iter, Int32(s.warm_start), s.stats))
    check(ccall((:tog_get_u, libtog), Cint, (Ptr{Cvoid}, Ptr{Float64}), s.handle, s.u))
    return nothing
end

# ComplianceFun(solver) builds cell_comp / grad from the grid only; its call is specialised here.
function (o::ComplianceFun{T,<:GB300FEASolver})(x::PseudoDensities) where {T}
    s = o.solver
    s.vars .= x.x
    s()
    c = Ref{Float64}(0.0)
    check(ccall((:tog_compliance, libtog), Cint, (Ptr{Cvoid}, Ref{Float64}, Ptr{Float64}), s.handle, c, o.grad))
    return c[]
end

# ---- multiple loads: MeanComplianceFun / BlockComplianceFun (src/Functions/mean_compliance.jl,
#      block_compliance.jl) on a GB300FEASolver.  The reference's versions need the per-element
#      Kes the GB300 solver never builds; these methods solve every rhs column on the device.
const TOF = TopOpt.Functions
function _multiload!(s::GB300FEASolver, cols::SparseMatrixCSC)
    length(s.vars) == getncells(s.problem) || throw(DimensionMismatch("vars"))
    check(ccall((:tog_set_vars, libtog), Cint, (Ptr{Cvoid}, Ptr{Float64}), s.handle, s.vars))
    c = zeros(size(cols, 2))
    colptr = Int64.(cols.colptr .- 1)
    rowval = Int32.(cols.rowval .- 1)
    nzval = Vector{Float64}(cols.nzval)
    check(ccall((:tog_multiload_compliance, libtog), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Int64}, Ptr{Int32}, Ptr{Float64}, Cint, Float64, Float64, Int32,
                 Ptr{Float64}, Ref{SolveStats}),
                s.handle, Int32(size(cols, 2)), colptr, rowval, nzval, s.precision, s.rtol, s.abstol,
                Int32(s.cg_max_iter), c, s.stats))
    return c
end
function _multiload_grad!(out, s::GB300FEASolver, w::AbstractVector)
    check(ccall((:tog_multiload_gradient, libtog), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}),
                s.handle, Int32(length(w)), Vector{Float64}(w), out))
    return out
end
_ml_columns(m::TOF.ExactMean, F) = (sparse(F), size(F, 2))
_ml_columns(m::TOF.ExactSVDMean, F) = (sparse(m.US), m.n)
function _ml_columns(m::TOF.TraceEstimationMean, F)
    m.sample_once || m.sample_method(m.V)
    return sparse(m.F * m.V), size(m.V, 2) * size(m.F, 2)
end
function _ml_columns(m::TOF.TraceEstimationSVDMean, F)
    m.sample_once || m.sample_method(m.V)
    return sparse(m.US * m.V), size(m.V, 2) * m.n
end
function (ec::TOF.MeanComplianceFun{T,<:ComplianceFun{T,<:GB300FEASolver}})(x::PseudoDensities) where {T}
    s = ec.compliance.solver
    s.vars .= x.x
    cols, n = _ml_columns(ec.method, ec.F)
    c = _multiload!(s, cols)
    _multiload_grad!(ec.grad, s, fill(1.0 / n, size(cols, 2)))
    return sum(c) / n
end
function TOF.compute_block_compliance(bc::TOF.BlockComplianceFun{T,<:ComplianceFun{T,<:GB300FEASolver}},
                                     m::TOF.ExactDiagonal) where {T}
    bc.raw_val .= _multiload!(bc.compliance.solver, sparse(m.F))
    return bc.raw_val
end
function TOF.compute_jtvp!_bc(out, bc::TOF.BlockComplianceFun{T,<:ComplianceFun{T,<:GB300FEASolver}},
                             m::TOF.ExactDiagonal, w) where {T}
    return _multiload_grad!(out, bc.compliance.solver, w)
end

function TopOpt.Functions.VolumeFun(s::GB300FEASolver{T}; fraction=true) where {T}
    rg = s.problem.rect_grid
    cellvolumes = fill(T(prod(rg.sizes)), getncells(s.problem))
    total = sum(cellvolumes)
    grad = fraction ? cellvolumes ./ total : copy(cellvolumes)
    return VolumeFun(s, cellvolumes, grad, total, fraction)
end

struct GB300DensityFilter{TS<:GB300FEASolver} <: AbstractDensityFilter
    solver::TS
    rmin::Float64
end
struct GB300SensFilter{TS<:GB300FEASolver} <: AbstractSensFilter
    solver::TS
    rmin::Float64
end

function _filter_setup(s::GB300FEASolver, rmin)
    check(ccall((:tog_filter_setup, libtog), Cint, (Ptr{Cvoid}, Float64), s.handle, Float64(rmin)))
end
function _filter_apply(s::GB300FEASolver, op::Integer, v::AbstractVector)
    out = similar(v, Float64)
    check(ccall((:tog_filter_apply, libtog), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}),
                s.handle, Int32(op), Vector{Float64}(v), out))
    return out
end

"""`DensityFilterFun(solver::GB300FEASolver; rmin)` (density_filter.jl:25-33)."""
function TopOpt.CheqFilters.DensityFilterFun(s::GB300FEASolver, rmin::Real, args...)
    _filter_setup(s, rmin)
    return GB300DensityFilter(s, Float64(rmin))
end
TopOpt.CheqFilters.DensityFilterFun(s::GB300FEASolver; rmin) = TopOpt.CheqFilters.DensityFilterFun(s, rmin)
function TopOpt.CheqFilters.SensFilterFun(s::GB300FEASolver, rmin::Real, args...)
    _filter_setup(s, rmin)
    return GB300SensFilter(s, Float64(rmin))
end
TopOpt.CheqFilters.SensFilterFun(s::GB300FEASolver; rmin) = TopOpt.CheqFilters.SensFilterFun(s, rmin)

(f::GB300DensityFilter)(x::PseudoDensities{I,P}) where {I,P} = PseudoDensities{I,P,true}(_filter_apply(f.solver, 0, x.x))
function ChainRulesCore.rrule(f::GB300DensityFilter, x::PseudoDensities)
    return f(x), Δ -> begin
        _Δ = ChainRulesCore.unthunk(Δ)
        _Δ = hasproperty(_Δ, :x) ? _Δ.x : _Δ
        (NoTangent(), Tangent{typeof(x)}(; x=_filter_apply(f.solver, 1, _Δ)))
    end
end
(f::GB300SensFilter)(x::PseudoDensities{I,P}) where {I,P} = PseudoDensities{I,P,true}(x.x)
function ChainRulesCore.rrule(f::GB300SensFilter, x::PseudoDensities)
    return x, Δ -> begin
        _Δ = ChainRulesCore.unthunk(Δ)
        _Δ = hasproperty(_Δ, :x) ? _Δ.x : _Δ
        (NoTangent(), Tangent{typeof(x)}(; x=_filter_apply(f.solver, 0, _Δ)))
    end
end

"""
    oc_update!(xnew, solver, x, dc, dv, w; volfrac, move=0.2) -> (change, λ)

Optimality-criteria update on the GPU (published OC method; TopOpt.jl has none).
"""
function oc_update!(xnew::Vector{Float64}, s::GB300FEASolver, x, dc, dv, w; volfrac, move=0.2)
    ch, lam = Ref(0.0), Ref(0.0)
    check(ccall((:tog_oc_update, libtog), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Float64, Float64,
                 Ptr{Float64}, Ref{Float64}, Ref{Float64}),
                s.handle, Vector{Float64}(x), Vector{Float64}(dc), Vector{Float64}(dv), Vector{Float64}(w),
                Float64(volfrac), Float64(move), xnew, ch, lam))
    return ch[], lam[]
end

_proj_kind(::TopOpt.Utilities.HeavisideProjectionFun) = Int32(1)
_proj_kind(::TopOpt.Utilities.SigmoidProjectionFun) = Int32(2)
function _project(s::GB300FEASolver, P, x::AbstractVector)
    y, dy = zeros(length(x)), zeros(length(x))
    check(ccall((:tog_projection, libtog), Cint,
                (Ptr{Cvoid}, Int32, Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                s.handle, _proj_kind(P), Float64(P.β), Vector{Float64}(x), y, dy))
    return y, dy
end

"""
    ProjectedDensityFilterFun(solver::GB300FEASolver; rmin, projection=HeavisideProjectionFun(10.0))
    GB300ProjectedDensityFilter(filter::GB300DensityFilter, preproj, postproj)

ProjectedDensityFilterFun (src/CheqFilters/density_filter.jl:129-169) on the device: the
reference type holds a concrete `DensityFilterFun`, so the GB300 filter comes with its own
wrapper.  The projections (Heaviside / sigmoid, `src/Utilities/penalties.jl:75-94`) run
through `tog_projection`; the rrule is the chain rule through both projections and J'.
"""
struct GB300ProjectedDensityFilter{TF<:GB300DensityFilter,TP1,TP2} <: AbstractDensityFilter
    filter::TF
    preproj::TP1
    postproj::TP2
end
function TopOpt.CheqFilters.ProjectedDensityFilterFun(s::GB300FEASolver; rmin,
                                                      projection=TopOpt.Utilities.HeavisideProjectionFun(10.0))
    return GB300ProjectedDensityFilter(TopOpt.CheqFilters.DensityFilterFun(s, rmin), nothing, projection)
end
function _projected_forward(f::GB300ProjectedDensityFilter, x::AbstractVector)
    s = f.filter.solver
    x1, d1 = f.preproj === nothing ? (Vector{Float64}(x), nothing) : _project(s, f.preproj, x)
    fx = _filter_apply(s, 0, x1)
    y, d2 = f.postproj === nothing ? (fx, nothing) : _project(s, f.postproj, fx)
    return y, d1, d2
end
(f::GB300ProjectedDensityFilter)(x::PseudoDensities{I,P}) where {I,P} =
    PseudoDensities{I,P,true}(_projected_forward(f, x.x)[1])
function ChainRulesCore.rrule(f::GB300ProjectedDensityFilter, x::PseudoDensities{I,P}) where {I,P}
    y, d1, d2 = _projected_forward(f, x.x)
    return PseudoDensities{I,P,true}(y), Δ -> begin
        _Δ = ChainRulesCore.unthunk(Δ)
        _Δ = hasproperty(_Δ, :x) ? _Δ.x : _Δ
        g = d2 === nothing ? Vector{Float64}(_Δ) : _Δ .* d2
        g = _filter_apply(f.filter.solver, 1, g)
        d1 === nothing || (g = g .* d1)
        (NoTangent(), Tangent{typeof(x)}(; x=g))
    end
end

"""
    GB300FixedElementProjector(solver, p::FixedElementProjectorFun)

FixedElementProjectorFun (src/Functions/fixed_element.jl:13-79) on the device of `solver`:
calling it projects x_free (black 1, white 0, free cells copied), its rrule gathers the
free cells' cotangent.  Constructing it sets the solver's active-element mask, so
`simp_step!` and `oc_update!` hold the fixed cells at their densities.
"""
struct GB300FixedElementProjector{TS<:GB300FEASolver}
    solver::TS
    proj::TopOpt.Functions.FixedElementProjectorFun
end
function GB300FixedElementProjector(s::GB300FEASolver, p::TopOpt.Functions.FixedElementProjectorFun)
    p.nel == getncells(s.problem) || throw(DimensionMismatch("projector and problem cell counts differ"))
    state = zeros(UInt8, p.nel)
    state[p.black] .= 0x01
    state[p.white] .= 0x02
    check(ccall((:tog_set_fixed_elements, libtog), Cint, (Ptr{Cvoid}, Ptr{UInt8}), s.handle, state))
    return GB300FixedElementProjector{typeof(s)}(s, p)
end
clear_fixed_elements!(s::GB300FEASolver) =
    check(ccall((:tog_set_fixed_elements, libtog), Cint, (Ptr{Cvoid}, Ptr{UInt8}), s.handle, C_NULL))
function (g::GB300FixedElementProjector)(x_free::AbstractVector)
    nf = count(g.proj.free)
    length(x_free) == nf || throw(ArgumentError(
        "x_free length ($(length(x_free))) must match number of free elements ($nf)"))
    ρ = zeros(g.proj.nel)
    check(ccall((:tog_fixed_element_project, libtog), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{Float64}),
                g.solver.handle, Vector{Float64}(x_free), Int64(nf), ρ))
    return ρ
end
function ChainRulesCore.rrule(g::GB300FixedElementProjector, x_free::AbstractVector)
    y = g(x_free)
    return y, Δ -> begin
        dx = zeros(count(g.proj.free))
        check(ccall((:tog_fixed_element_pullback, libtog), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
                    g.solver.handle, Vector{Float64}(ChainRulesCore.unthunk(Δ)), dx))
        (NoTangent(), dx)
    end
end

"""
    mma_update!(xnew, solver, x, df0, g, dg; move=0.5) -> (change, λ)
    mma_reset!(solver)

One step of MMA (Svanberg's method of moving asymptotes, what `optimize(model, MMA87(), x0)`
runs in the reference's SIMP scripts) on the GPU for min f s.t. g(x) <= 0 on [0, 1]^n.
The asymptotes and the last two iterates stay in the solver's handle between calls.
"""
function mma_update!(xnew::Vector{Float64}, s::GB300FEASolver, x, df0, g::Real, dg; move=0.5)
    ch, lam = Ref(0.0), Ref(0.0)
    check(ccall((:tog_mma_update, libtog), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Float64, Ptr{Float64}, Float64, Ptr{Float64},
                 Ref{Float64}, Ref{Float64}),
                s.handle, Vector{Float64}(x), Vector{Float64}(df0), Float64(g), Vector{Float64}(dg), Float64(move),
                xnew, ch, lam))
    return ch[], lam[]
end
mma_reset!(s::GB300FEASolver) = check(ccall((:tog_mma_reset, libtog), Cint, (Ptr{Cvoid},), s.handle))

mutable struct IterStats
    compliance::Float64
    volume::Float64
    change::Float64
    lambda::Float64
    cg_iterations::Int32
    outer_iterations::Int32
    oc_steps::Int32
    status::Int32
    rel_residual::Float64
end
IterStats() = IterStats(0, 0, 0, 0, 0, 0, 0, 0, 0)

"""
    simp_init!(solver, x0; volfrac, rmin, filter=:density, move=nothing, optimizer=:oc)
    simp_step!(solver) -> IterStats

Device-resident SIMP loop: one call per design iteration, the design stays in HBM.
`optimizer` is `:oc` (move limit 0.2 unless `move` is given) or `:mma` (the volume
constraint through MMA, move limit 0.5 unless given).
"""
function simp_init!(s::GB300FEASolver, x0::AbstractVector; volfrac, rmin=0.0, filter=:density, move=nothing,
                    optimizer=:oc)
    kind = filter === :density ? Int32(1) : filter === :sens ? Int32(2) : Int32(0)
    opt = optimizer === :mma ? Int32(1) : Int32(0)
    check(ccall((:tog_simp_set_optimizer, libtog), Cint, (Ptr{Cvoid}, Int32, Float64), s.handle, opt,
                optimizer === :mma && move !== nothing ? Float64(move) : 0.0))
    ocmove = optimizer === :oc && move !== nothing ? Float64(move) : 0.2
    check(ccall((:tog_simp_init, libtog), Cint, (Ptr{Cvoid}, Int32, Float64, Float64, Float64, Ptr{Float64}),
                s.handle, kind, Float64(rmin), Float64(volfrac), ocmove, Vector{Float64}(x0)))
end
function simp_step!(s::GB300FEASolver)
    st = Ref(IterStats())
    check(ccall((:tog_simp_step, libtog), Cint, (Ptr{Cvoid}, Cint, Float64, Int32, Int32, Ref{IterStats}),
                s.handle, s.precision, s.rtol, Int32(s.cg_max_iter), Int32(s.warm_start), st))
    return st[]
end
function design(s::GB300FEASolver)
    x = zeros(getncells(s.problem))
    check(ccall((:tog_get_design, libtog), Cint, (Ptr{Cvoid}, Ptr{Float64}), s.handle, x))
    return x
end

# --------------------------------------------------------------------------- batched 2D
mutable struct BatchStats
    steps::Int32
    pcg_loops::Int32
    failed::Int32
    reliable_updates::Int32
end
BatchStats() = BatchStats(0, 0, 0, 0)

"""
    BatchedSIMP(nelx, nely, load_j, volfrac, rmin; rtol=1e-8, E=1.0, nu=0.3, xmin=1e-9, p=3.0)

Many independent 2D cantilevers (left edge clamped, unit load [0, -1] at node (nelx, load_j)),
each design iteration of all of them one CUDA graph launch (no TopOpt.jl counterpart: there a
user loops over problems).  `autotune!`, `batch_step!`, `batch_results`.
"""
mutable struct BatchedSIMP
    handle::Ptr{Cvoid}
    n::Int
end
function BatchedSIMP(nelx, nely, load_j, volfrac, rmin; rtol=1e-8, E=1.0, nu=0.3, xmin=1e-9, p=3.0)
    n = length(nelx)
    desc = ProblemDesc(Int32(2), (Int32(0), Int32(0), Int32(0)), (1.0, 1.0, 1.0), E, nu, Int32(0), xmin, p)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:tog_batch_create, libtog), Cint,
                (Int32, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Ptr{Float64}, Ref{ProblemDesc}, Float64,
                 Int32, Ref{Ptr{Cvoid}}),
                n, Int32.(nelx), Int32.(nely), Int32.(load_j), Float64.(volfrac), Float64.(rmin), desc, rtol, 0, h))
    b = BatchedSIMP(h[], n)
    finalizer(b) do x
        x.handle == C_NULL || ccall((:tog_batch_destroy, libtog), Cint, (Ptr{Cvoid},), x.handle)
    end
    return b
end
function autotune!(b::BatchedSIMP)
    rows = Ref{Int32}(0)
    check(ccall((:tog_batch_autotune, libtog), Cint, (Ptr{Cvoid}, Ref{Int32}), b.handle, rows))
    return rows[]
end
function batch_step!(b::BatchedSIMP)
    st = Ref(BatchStats())
    check(ccall((:tog_batch_step, libtog), Cint, (Ptr{Cvoid}, Ref{BatchStats}), b.handle, st))
    return st[]
end
function batch_results(b::BatchedSIMP)
    c, ch, it = zeros(b.n), zeros(b.n), zeros(Int32, b.n)
    check(ccall((:tog_batch_results, libtog), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}),
                b.handle, c, ch, it))
    return c, ch, it
end

# --------------------------------------------------------------------------- learned warm start
"""
    WarmStartNet(nodes; seed=0, params=nothing)

The learned warm-start network of the library (tensor-core conv3d encoder-decoder) for a 3D
node grid `nodes = (nnx, nny, nnz)`, optionally loaded with a trained FP32 parameter vector.
`attach_network!(solver, net)` then makes `simp_step!` start from the Galerkin-corrected
previous displacement when the solver's `warm_start` is 2 (no TopOpt.jl counterpart).
"""
mutable struct WarmStartNet
    handle::Ptr{Cvoid}
end
function WarmStartNet(nodes; seed=0, params=nothing)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:tog_nn_create, libtog), Cint, (Ptr{Int32}, Int32, UInt64, Ref{Ptr{Cvoid}}),
                Int32.(collect(nodes)), Int32(1), UInt64(seed), h))
    net = WarmStartNet(h[])
    finalizer(net) do x
        x.handle == C_NULL || ccall((:tog_nn_destroy, libtog), Cint, (Ptr{Cvoid},), x.handle)
    end
    if params !== nothing
        check(ccall((:tog_nn_set_params, libtog), Cint, (Ptr{Cvoid}, Ptr{Float32}), net.handle, Float32.(params)))
    end
    return net
end
function attach_network!(s::GB300FEASolver, net::WarmStartNet)
    check(ccall((:tog_set_warm_start_net, libtog), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), s.handle, net.handle))
    return s
end

end # module
