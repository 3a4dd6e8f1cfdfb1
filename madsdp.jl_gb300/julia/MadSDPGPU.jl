# Julia binding of libmadsdp_gpu.so (include/madsdp_gpu.h).
#
# Drops in beside MadSDP's CPU components: the same component values
# (MadSDP.NT(), MadSDP.EigenStep(), MadSDP.Mehrotra(), MadSDP.DenseCholesky(),
# ...) select the device kernel, and `MadSDPGPU.Solver` can replace
# `MadSDP.Solver` as the SolverCore solver behind `LowRankOpt.Optimizer`
# (the role of src/moi.jl:42-93).  Requires the library built with
# `python madsdp.jl_gb300/build.py`; set ENV["MADSDP_GPU_LIB"] to its path.
module MadSDPGPU

import LowRankOpt as LRO
import MadNLP
import MadSDP
import SolverCore
import SparseArrays

const LIB = get(ENV, "MADSDP_GPU_LIB", joinpath(@__DIR__, "..", "lib", "libmadsdp_gpu.so"))

struct Components
    algorithm::Int32; direction::Int32; step::Int32; centering::Int32
    initial_point::Int32; schur::Int32; precision::Int32; centering_max_iter::Int32
    tau::Float64; shrink::Float64; boundary::Float64; sigma_exponent::Float64
    initial_ratio::Float64; ratio::Float64; scale::Float64; initial_shift::Float64
    max_shift::Float64; dc_beta::Float64; dc_delta::Float64; dc_A::Float64
end

struct Options
    tol::Float64; max_iter::Int32; max_schur_reg::Int32; max_wall_time::Float64
    mu_min::Float64; regularize_schur::Float64; datasparsity::Int32; mixed_refine::Int32
    switch_tol::Float64
end

struct ProblemDesc
    nblocks::Int32; m::Int32; ns::Int32; pad0::Int32
    sides::Ptr{Int32}; C::Ptr{Ptr{Float64}}; A_nnz::Ptr{Int64}
    A_con::Ptr{Ptr{Int32}}; A_row::Ptr{Ptr{Int32}}; A_col::Ptr{Ptr{Int32}}
    A_val::Ptr{Ptr{Float64}}; b::Ptr{Float64}; d_lin::Ptr{Float64}; C_lin::Ptr{Float64}
end

struct Stats
    status::Int32; iter::Int32; iter_fp32::Int32; iter_fp64::Int32
    pobj::Float64; dobj::Float64; inf_pr::Float64; inf_du::Float64; gap::Float64
    mu::Float64; sigma::Float64; alpha::Float64; beta::Float64; solve_ns::Float64
    n_newton::Int32; n_predictor::Int32
end

function check(ctx, rc, what)
    rc == 0 && return
    msg = unsafe_string(ccall((:msdp_last_error, LIB), Cstring, (Ptr{Cvoid},), ctx))
    rc == -1 && throw(ArgumentError(msg))            # invalid configuration
    rc == -5 && error(msg)                           # no initial point (ErrorException)
    error("$what failed ($rc): $msg")
end

# Component values -> the C selector struct (defaults of src/components.jl).
function components(; algorithm, direction, step, centering, initial_point, schur, precision)
    c = Ref{Components}()
    ccall((:msdp_default_components, LIB), Cvoid, (Ptr{Components},), c)
    x = c[]
    alg = algorithm isa MadSDP.DualCentering ? Int32(1) : Int32(0)
    dir = direction isa MadSDP.HKM ? Int32(1) : Int32(0)
    stp = step isa MadSDP.CholeskyBacktrack ? Int32(1) : Int32(0)
    cen = centering isa MadSDP.AdaptiveMu ? Int32(1) : Int32(0)
    ip = initial_point isa MadSDP.InitialPoint ? Int32(1) : initial_point isa MadSDP.DualShift ? Int32(2) : Int32(0)
    sch = schur isa MadSDP.QRSchur ? Int32(2) : schur isa MadSDP.MadNLPSchur ? Int32(1) : Int32(0)
    tau = step isa MadSDP.EigenStep ? Float64(step.τ) : x.tau
    shrink, boundary = step isa MadSDP.CholeskyBacktrack ? (Float64(step.shrink), Float64(step.boundary)) : (x.shrink, x.boundary)
    sexp = centering isa MadSDP.Mehrotra ? Float64(centering.σ_exponent) : x.sigma_exponent
    ir, r = centering isa MadSDP.AdaptiveMu ? (Float64(centering.initial_ratio), Float64(centering.ratio)) : (x.initial_ratio, x.ratio)
    scale = initial_point isa MadSDP.ScaledIdentity && !isnothing(initial_point.scale) ? Float64(initial_point.scale) : 0.0
    ish, msh = initial_point isa MadSDP.DualShift ? (Float64(initial_point.initial_shift), Float64(initial_point.max_shift)) : (x.initial_shift, x.max_shift)
    return Components(alg, dir, stp, cen, ip, sch, precision === :mixed ? Int32(1) : precision === :fp64_tensor ? Int32(2) : Int32(0),
                      x.centering_max_iter, tau, shrink, boundary, sexp, ir, r, scale, ish, msh,
                      x.dc_beta, x.dc_delta, x.dc_A)
end

# Full symmetric coordinate list of the constraint matrices of block i.
function coordinates(model::LRO.Model, i, m)
    con, row, col, val = Int32[], Int32[], Int32[], Float64[]
    for j in 1:m
        A = LRO.jac(model, j, LRO.MatrixIndex(i))
        S = SparseArrays.sparse(A)
        rows, vals = SparseArrays.rowvals(S), SparseArrays.nonzeros(S)
        for c in axes(S, 2), p in SparseArrays.nzrange(S, c)
            push!(con, j - 1); push!(row, rows[p] - 1); push!(col, c - 1); push!(val, vals[p])
        end
    end
    return con, row, col, val
end

"""
    solve(model::LRO.Model; direction, step, centering, algorithm, initial_point,
          schur, precision = :fp64, device = 0, options...)

Solve `model` on the GPU with the given MadSDP components; returns the
stats (status as `MadNLP.Status`), X blocks, y, x and z.
"""
function solve(model::LRO.Model; direction = MadSDP.NT(), step = MadSDP.EigenStep(),
               centering = MadSDP.Mehrotra(), algorithm = MadSDP.PrimalDual(direction, step, centering),
               initial_point = MadSDP.default_initial_point(algorithm), schur = MadSDP.DenseCholesky(),
               precision = :fp64, device = 0, engine = :auto, options...)
    nb, ns, m = LRO.num_matrices(model), LRO.num_scalars(model), model.meta.ncon
    sides = Int32[LRO.side_dimension(model, LRO.MatrixIndex(i)) for i in 1:nb]
    Cs = [Matrix{Float64}(LRO.grad(model, LRO.MatrixIndex(i))) for i in 1:nb]
    coords = [coordinates(model, i, m) for i in 1:nb]
    b = Vector{Float64}(LRO.cons_constant(model))
    d = Vector{Float64}(model.d_lin)
    Cl = Matrix{Float64}(model.C_lin)
    # the pointer arrays are named so that GC.@preserve keeps them alive
    Cp = [pointer(c) for c in Cs]
    nnz = Int64[length(c[4]) for c in coords]
    conp, rowp = [pointer(c[1]) for c in coords], [pointer(c[2]) for c in coords]
    colp, valp = [pointer(c[3]) for c in coords], [pointer(c[4]) for c in coords]
    GC.@preserve sides Cs coords b d Cl Cp nnz conp rowp colp valp begin
        desc = ProblemDesc(nb, m, ns, 0, pointer(sides), pointer(Cp), pointer(nnz),
                           pointer(conp), pointer(rowp), pointer(colp), pointer(valp),
                           pointer(b), pointer(d), pointer(Cl))
        opt = Ref{Options}()
        ccall((:msdp_default_options, LIB), Cvoid, (Ptr{Options},), opt)
        o = opt[]
        kw = Dict(options)
        o = Options(get(kw, :tol, o.tol), get(kw, :max_iter, o.max_iter), get(kw, :max_schur_reg, o.max_schur_reg),
                    get(kw, :max_wall_time, o.max_wall_time), get(kw, :mu_min, o.mu_min),
                    get(kw, :regularize_schur, o.regularize_schur), o.datasparsity, o.mixed_refine, o.switch_tol)
        comp = components(; algorithm, direction, step, centering, initial_point, schur, precision)
        ctx = Ref{Ptr{Cvoid}}(C_NULL)
        check(C_NULL, ccall((:msdp_context_create, LIB), Cint, (Cint, Ptr{Ptr{Cvoid}}), device, ctx), "context")
        if engine == :instance || precision === :fp64_tensor || (engine == :auto && (maximum(sides; init = 0) > 64 || m > 300))
            # one large problem on the whole GPU (msdp_solver_*)
            sv = Ref{Ptr{Cvoid}}(C_NULL)
            rc = ccall((:msdp_solver_create, LIB), Cint,
                       (Ptr{Cvoid}, Ref{ProblemDesc}, Ref{Components}, Ref{Options}, Ptr{Ptr{Cvoid}}),
                       ctx[], desc, comp, o, sv)
            check(ctx[], rc, "msdp_solver_create")
            if initial_point isa MadSDP.InitialPoint
                Xs = [Matrix{Float64}(X) for X in initial_point.X]
                y0 = Vector{Float64}(initial_point.y)
                x0 = isnothing(initial_point.x) ? nothing : Vector{Float64}(initial_point.x)
                GC.@preserve Xs y0 x0 check(ctx[], ccall((:msdp_solver_set_initial_point, LIB), Cint,
                                   (Ptr{Cvoid}, Ptr{Ptr{Float64}}, Ptr{Float64}, Ptr{Float64}),
                                   sv[], [pointer(X) for X in Xs], y0, isnothing(x0) ? C_NULL : pointer(x0)),
                      "initial point")
            end
            check(ctx[], ccall((:msdp_solver_solve, LIB), Cint, (Ptr{Cvoid},), sv[]), "msdp_solver_solve")
            st = Ref{Stats}()
            check(ctx[], ccall((:msdp_solver_get_stats, LIB), Cint, (Ptr{Cvoid}, Ptr{Stats}), sv[], st), "stats")
            X = [zeros(n, n) for n in sides]
            y, x, z = zeros(m), zeros(ns), zeros(ns)
            check(ctx[], ccall((:msdp_solver_get_solution, LIB), Cint,
                               (Ptr{Cvoid}, Ptr{Ptr{Float64}}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                               sv[], [pointer(Xi) for Xi in X], y, x, z), "solution")
            ccall((:msdp_solver_destroy, LIB), Cint, (Ptr{Cvoid},), sv[])
            ccall((:msdp_context_destroy, LIB), Cint, (Ptr{Cvoid},), ctx[])
            return (stats = st[], status = MadNLP.Status(st[].status), X = X, y = y, x = x, z = z)
        end
        batch = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:msdp_batch_create, LIB), Cint,
                   (Ptr{Cvoid}, Ref{ProblemDesc}, Int32, Ref{Components}, Ref{Options}, Ptr{Ptr{Cvoid}}),
                   ctx[], desc, 1, comp, o, batch)
        check(ctx[], rc, "msdp_batch_create")
        if initial_point isa MadSDP.InitialPoint
            Xs = [Matrix{Float64}(X) for X in initial_point.X]
            y0 = Vector{Float64}(initial_point.y)
            x0 = isnothing(initial_point.x) ? nothing : Vector{Float64}(initial_point.x)
            GC.@preserve Xs y0 x0 check(ctx[], ccall((:msdp_batch_set_initial_point, LIB), Cint,
                               (Ptr{Cvoid}, Int32, Ptr{Ptr{Float64}}, Ptr{Float64}, Ptr{Float64}),
                               batch[], 0, [pointer(X) for X in Xs], y0, isnothing(x0) ? C_NULL : pointer(x0)),
                  "initial point")
        end
        check(ctx[], ccall((:msdp_batch_solve, LIB), Cint, (Ptr{Cvoid},), batch[]), "msdp_batch_solve")
        st = Ref{Stats}()
        check(ctx[], ccall((:msdp_batch_get_stats, LIB), Cint, (Ptr{Cvoid}, Int32, Ptr{Stats}), batch[], 0, st), "stats")
        X = [zeros(n, n) for n in sides]
        y, x, z = zeros(m), zeros(ns), zeros(ns)
        check(ctx[], ccall((:msdp_batch_get_solution, LIB), Cint,
                           (Ptr{Cvoid}, Int32, Ptr{Ptr{Float64}}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                           batch[], 0, [pointer(Xi) for Xi in X], y, x, z), "solution")
        ccall((:msdp_batch_destroy, LIB), Cint, (Ptr{Cvoid},), batch[])
        ccall((:msdp_context_destroy, LIB), Cint, (Ptr{Cvoid},), ctx[])
        return (stats = st[], status = MadNLP.Status(st[].status), X = X, y = y, x = x, z = z)
    end
end

"""
    Solver(model::LRO.Model; kws...)

SolverCore wrapper with the role of `MadSDP.Solver` (src/moi.jl:42-72):
`LowRankOpt.Optimizer` creates it and calls `SolverCore.solve!`, which runs
the device path with the components given as raw attributes.
"""
mutable struct Solver{T,M} <: SolverCore.AbstractOptimizationSolver
    model::M
    result::Any
    stats::SolverCore.GenericExecutionStats{T,Vector{T},Vector{T},Any}
end

Solver(model::LRO.AbstractModel{T}; kws...) where {T} =
    Solver{T,typeof(model)}(model, nothing, SolverCore.GenericExecutionStats(model))

function SolverCore.solve!(s::Solver, ::Any; verbose::Int = 1, kws...)
    model = s.model isa LRO.BufferedModelForSchur ? s.model.model : s.model
    r = solve(model; kws...)
    s.result = r
    SolverCore.set_status!(s.stats, MadSDP._solvercore_status(r.status))
    SolverCore.set_objective!(s.stats, r.stats.pobj)
    SolverCore.set_solver_specific!(s.stats, :dual_objective, r.stats.dobj)
    SolverCore.set_constraint_multipliers!(s.stats, copy(r.y))
    SolverCore.set_residuals!(s.stats, r.stats.inf_pr, r.stats.inf_du)
    SolverCore.set_iter!(s.stats, r.stats.iter)
    return s.stats
end

# The primal solution as LowRankOpt expects it (src/moi.jl:76-78).
import MathOptInterface as MOI
MOI.get(s::Solver, ::LRO.Solution) = LRO.ShapedSolution(copy(s.result.x), [copy(X) for X in s.result.X])
MOI.get(::Solver, ::MOI.SolverName) = "MadSDPGPU"

end # module
