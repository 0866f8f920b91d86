# Julia glue for libgbcycle.so: GB300 Green's functions and a drop-in ODE right-hand side for
# Oetqf.jl. The reference's mesh, property and assemble API stays as it is; `assemble_gb300`
# returns an ODEProblem{true} whose f(du, u, p, t) calls the CUDA RHS through ccall.
# (Not exercised in this repository's tests: no Julia toolchain is available where they run.)
module OetqfGB300

using Oetqf, RecursiveArrayTools, OrdinaryDiffEq

const libgbc = get(ENV, "GBCYCLE_LIB", joinpath(@__DIR__, "..", "lib", "libgbcycle.so"))

struct GbcFaultMesh
    nx::Cint; nxi::Cint
    x::Ptr{Cdouble}; xi::Ptr{Cdouble}; y::Ptr{Cdouble}; z::Ptr{Cdouble}
    ax::Ptr{Cdouble}; axi::Ptr{Cdouble}
    dx::Cdouble; dxi::Cdouble; dep::Cdouble; dip::Cdouble
end

struct GbcHexMesh
    ne::Cint
    cx::Ptr{Cdouble}; cy::Ptr{Cdouble}; cz::Ptr{Cdouble}
    qx::Ptr{Cdouble}; qy::Ptr{Cdouble}; qz::Ptr{Cdouble}
    dx::Ptr{Cdouble}; dy::Ptr{Cdouble}; dz::Ptr{Cdouble}
end

function check(rc)
    rc == 0 && return
    buf = Vector{UInt8}(undef, 1024)
    ccall((:gbc_last_error, libgbc), Cint, (Ptr{UInt8}, Csize_t), buf, length(buf))
    throw(ErrorException("gbcycle error $rc: " * unsafe_string(pointer(buf))))
end

pairs_rowmajor(a) = collect(Iterators.flatten(a))   # Vector{NTuple{2}} -> (n,2) row-major

"GPU stress_greens_function(mesh::RectOkadaMesh, λ, μ; ...) (src/BEM/GF.jl:31)."
function stress_greens_function_gb300(mf::RectOkadaMesh, λ::Float64, μ::Float64;
        ftype=StrikeSlip(), fourier::Bool=true, nrept::Integer=2, buffer_ratio::Real=0)
    ax, axi = pairs_rowmajor(mf.ax), pairs_rowmajor(mf.aξ)
    GC.@preserve mf ax axi begin
        m = GbcFaultMesh(mf.nx, mf.nξ, pointer(mf.x), pointer(mf.ξ), pointer(mf.y), pointer(mf.z),
                         pointer(ax), pointer(axi), mf.Δx, mf.Δξ, mf.dep, mf.dip)
        out = fourier ? Array{ComplexF64}(undef, mf.nx, mf.nξ, mf.nξ) : Array{Float64}(undef, mf.nx, mf.nξ, mf.nξ)
        check(ccall((:gbc_stress_gf_ff, libgbc), Cint,
                    (Ref{GbcFaultMesh}, Cdouble, Cdouble, Cint, Cint, Cint, Cdouble, Ptr{Cvoid}),
                    m, λ, μ, ftype isa StrikeSlip ? 0 : 1, fourier, nrept, buffer_ratio, out))
    end
    return out
end

mutable struct GB300Model
    h::Ptr{Cvoid}
    nx::Int; nξ::Int; ne::Int
end

function GB300Model(nx, nξ, ne=0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gbc_model_create, libgbc), Cint, (Cint, Cint, Cint, Ref{Ptr{Cvoid}}), nx, nξ, ne, h))
    m = GB300Model(h[], nx, nξ, ne)
    finalizer(x -> ccall((:gbc_model_destroy, libgbc), Cvoid, (Ptr{Cvoid},), x.h), m)
    return m
end

set_gf!(m::GB300Model, which::Integer, gf::AbstractArray) =
    check(ccall((:gbc_model_set_gf, libgbc), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}), m.h, which, gf))

function set_props!(m::GB300Model, p::RateStateQuasiDynamicProperty)
    check(ccall((:gbc_model_set_fault_props, libgbc), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble),
                m.h, p.a, p.b, p.L, p.σ, p.η, p.vpl, p.f₀, p.v₀))
end

function set_props!(m::GB300Model, p::PowerLawViscosityProperty)
    check(ccall((:gbc_model_set_mantle_props, libgbc), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                m.h, Vector{Float64}(p.γ), Vector{Float64}(p.n), Vector{Float64}(p.dϵ₀)))
end

"CompositePowerLawViscosityProperty (property.jl:43-48): the laws stacked law-major."
function set_props!(m::GB300Model, p::CompositePowerLawViscosityProperty)
    γ = reduce(vcat, (Vector{Float64}(q.γ) for q in p.piter))
    n = reduce(vcat, (Vector{Float64}(q.n) for q in p.piter))
    check(ccall((:gbc_model_set_mantle_props_composite, libgbc), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                m.h, length(p.piter), γ, n, Vector{Float64}(p.dϵ₀)))
end

"DilatancyProperty (property.jl:27-32) of a fault-only model; its state is (v, θ, δ, 𝓅)."
function set_props!(m::GB300Model, p::DilatancyProperty)
    check(ccall((:gbc_model_set_dilatancy, libgbc), Cint,
                (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                m.h, Vector{Float64}(vec(p.tₚ)), Vector{Float64}(vec(p.ϵ)), Vector{Float64}(vec(p.β)),
                Vector{Float64}(vec(p.p₀))))
end

"The drop-in derivative: OrdinaryDiffEq calls f(du, u, p, t) in place; u and du are ArrayPartitions."
function gpu_ode(du::ArrayPartition, u::ArrayPartition, m::GB300Model, t)
    n = length(u.x)
    up = Ptr{Cdouble}[pointer(x) for x in u.x]
    dp = Ptr{Cdouble}[pointer(x) for x in du.x]
    GC.@preserve u du up dp begin
        check(ccall((:gbc_rhs, libgbc), Cint, (Ptr{Cvoid}, Cdouble, Ptr{Ptr{Cdouble}}, Ptr{Ptr{Cdouble}}, Cint),
                    m.h, t, up, dp, n))
    end
    return nothing
end

struct GbcSolverOpts
    reltol::Cdouble; abstol::Cdouble; dt0::Cdouble; dtmax::Cdouble; dtmin::Cdouble
    maxiters::Clonglong
    alg::Cint
end

mutable struct GbcSolverStats
    naccept::Clonglong; nreject::Clonglong; nrhs::Clonglong
    t::Cdouble; dt::Cdouble
    status::Cint
end

"""
    solve_gb300(prob, alg; reltol, abstol, dt, dtmax, maxiters)

`solve(prob, alg; ...)` (src/io.jl:125-130) with the whole integration on the device: `VCABM5()` or
`Tsit5()` with the same options; returns (u(t_end) as an ArrayPartition like `prob.u0`, stats).
"""
function solve_gb300(prob::ODEProblem, alg; reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=Inf, dtmin=1e-14,
                     maxiters::Integer=10^9)
    m = prob.p::GB300Model
    code = alg isa VCABM5 ? Cint(1) : alg isa Tsit5 ? Cint(0) : throw(ArgumentError("VCABM5() or Tsit5()"))
    o = GbcSolverOpts(reltol, abstol, dt, isfinite(dtmax) ? dtmax : 1e300, dtmin, maxiters, code)
    st = GbcSolverStats(0, 0, 0, 0.0, 0.0, 0)
    u = reduce(vcat, (vec(copy(x)) for x in prob.u0.x))
    rc = ccall((:gbc_integrate, libgbc), Cint,
               (Ptr{Cvoid}, Ptr{Cdouble}, Cdouble, Cdouble, Ref{GbcSolverOpts}, Ref{GbcSolverStats}),
               m.h, u, prob.tspan[1], prob.tspan[2], o, st)
    rc == 0 || rc == -5 || check(rc)
    out = deepcopy(prob.u0)
    off = 0
    for x in out.x
        copyto!(x, 1, u, off + 1, length(x)); off += length(x)
    end
    return out, st
end

"assemble(gf, p, u0, tspan) with the RHS on the GB300 (src/BEM/equation.jl:81-89)."
function assemble_gb300(gf::AbstractArray, p::RateStateQuasiDynamicProperty, u0::ArrayPartition, tspan::NTuple{2})
    nx, nξ = size(u0.x[1])
    m = GB300Model(nx, nξ, 0)
    set_gf!(m, eltype(gf) <: Complex ? 1 : 0, gf)
    set_props!(m, p)
    return ODEProblem{true}(gpu_ode, u0, tspan, m)
end

"assemble(gf₁₁, gf₁₂, gf₂₁, gf₂₂, pf, pa, u0, tspan) with the RHS on the GB300 (equation.jl:141-154)."
function assemble_gb300(gf₁₁::AbstractArray, gf₁₂::AbstractMatrix, gf₂₁::AbstractMatrix, gf₂₂::AbstractMatrix,
                        pf::RateStateQuasiDynamicProperty, pa::PowerLawViscosityProperty,
                        u0::ArrayPartition, tspan::NTuple{2})
    nx, nξ = size(u0.x[1]); ne = size(u0.x[3], 1)
    m = GB300Model(nx, nξ, ne)
    set_gf!(m, eltype(gf₁₁) <: Complex ? 1 : 0, gf₁₁)
    set_gf!(m, 2, gf₁₂); set_gf!(m, 3, gf₂₁); set_gf!(m, 4, gf₂₂)
    set_props!(m, pf); set_props!(m, pa)
    return ODEProblem{true}(gpu_ode, u0, tspan, m)
end

"""
Many property sets on one assembled geometry (the example's rerun of saved Green's functions with
other properties, examples/otf-with-mantle.jl:44-56, 140-162) integrated together: the variants share
`base`'s block-scaled BF16 Green's functions (`gbc_model_set_precision(base, 1)` first) and every
right-hand side is one tensor-core product over all variants' states.
"""
# gbc_solver_stats as an isbits struct, for arrays of them
struct GbcStatsC
    naccept::Clonglong; nreject::Clonglong; nrhs::Clonglong
    t::Cdouble; dt::Cdouble
    status::Cint
end

mutable struct GB300Sweep
    h::Ptr{Cvoid}
    base::GB300Model
    nvariants::Int
end

function GB300Sweep(base::GB300Model, nvariants::Integer)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gbc_sweep_create, libgbc), Cint, (Ptr{Cvoid}, Cint, Ref{Ptr{Cvoid}}), base.h, nvariants, h))
    s = GB300Sweep(h[], base, nvariants)
    finalizer(x -> ccall((:gbc_sweep_destroy, libgbc), Cvoid, (Ptr{Cvoid},), x.h), s)
    return s
end

function set_props!(s::GB300Sweep, k::Integer, p::RateStateQuasiDynamicProperty)
    check(ccall((:gbc_sweep_set_fault_props, libgbc), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble),
                s.h, k - 1, p.a, p.b, p.L, p.σ, p.η, p.vpl, p.f₀, p.v₀))
end

function set_props!(s::GB300Sweep, k::Integer, p::PowerLawViscosityProperty)
    check(ccall((:gbc_sweep_set_mantle_props, libgbc), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                s.h, k - 1, Vector{Float64}(p.γ), Vector{Float64}(p.n), Vector{Float64}(p.dϵ₀)))
end

"Integrates every variant's state (columns of `U`, each the flattened ArrayPartition) from t0 to t1."
function solve_gb300(s::GB300Sweep, U::Matrix{Float64}, t0, t1, alg; reltol=1e-6, abstol=1e-8, dt=1e-8, dtmax=Inf,
                     dtmin=1e-14, maxiters::Integer=10^9)
    size(U, 2) == s.nvariants || throw(DimensionMismatch("one column per variant"))
    code = alg isa VCABM5 ? Cint(1) : alg isa Tsit5 ? Cint(0) : throw(ArgumentError("VCABM5() or Tsit5()"))
    o = GbcSolverOpts(reltol, abstol, dt, isfinite(dtmax) ? dtmax : 1e300, dtmin, maxiters, code)
    st = Vector{GbcStatsC}(undef, s.nvariants)  # a C array of gbc_solver_stats
    out = copy(U)
    rc = ccall((:gbc_sweep_integrate, libgbc), Cint,
               (Ptr{Cvoid}, Ptr{Cdouble}, Cdouble, Cdouble, Ref{GbcSolverOpts}, Ptr{GbcStatsC}),
               s.h, out, t0, t1, o, st)
    rc == 0 || rc == -5 || check(rc)
    return out, st
end

"""
Many fault-only models of uneven size, each with its own mesh, properties, initial state and time
span, integrated in one persistent launch: per-model step control, large models split over
thread-block clusters and re-planned onto larger clusters as others finish (`gbc_ensemble_*`). The
batched counterpart of `solve(assemble(gf, p, u0, tspan), alg)` (src/BEM/equation.jl:81-89,
src/io.jl:125-130) called on each model in turn.
"""
mutable struct GB300Ensemble
    h::Ptr{Cvoid}
    nmodels::Int
end

function GB300Ensemble(meshes::AbstractVector{<:RectOkadaMesh})
    nx = Cint[mf.nx for mf in meshes]
    nξ = Cint[mf.nξ for mf in meshes]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gbc_ensemble_create, libgbc), Cint, (Cint, Ptr{Cint}, Ptr{Cint}, Ref{Ptr{Cvoid}}),
                length(meshes), nx, nξ, h))
    e = GB300Ensemble(h[], length(meshes))
    finalizer(x -> ccall((:gbc_ensemble_destroy, libgbc), Cvoid, (Ptr{Cvoid},), x.h), e)
    return e
end

"Model k's fault Green's function assembled on the device (stress_greens_function, src/BEM/GF.jl:31)."
function assemble!(e::GB300Ensemble, k::Integer, mf::RectOkadaMesh, λ::Float64, μ::Float64;
                   ftype=StrikeSlip(), nrept::Integer=2, buffer_ratio::Real=0)
    ax, axi = pairs_rowmajor(mf.ax), pairs_rowmajor(mf.aξ)
    GC.@preserve mf ax axi begin
        m = GbcFaultMesh(mf.nx, mf.nξ, pointer(mf.x), pointer(mf.ξ), pointer(mf.y), pointer(mf.z),
                         pointer(ax), pointer(axi), mf.Δx, mf.Δξ, mf.dep, mf.dip)
        check(ccall((:gbc_ensemble_assemble, libgbc), Cint,
                    (Ptr{Cvoid}, Cint, Ref{GbcFaultMesh}, Cdouble, Cdouble, Cint, Cint, Cdouble),
                    e.h, k - 1, m, λ, μ, ftype isa StrikeSlip ? 0 : 1, nrept, buffer_ratio))
    end
end

"Model k's fault Green's function from a host array: real (nx, nξ, nξ) or the rFFT form."
function set_gf!(e::GB300Ensemble, k::Integer, gf::AbstractArray)
    g = Array(gf)
    check(ccall((:gbc_ensemble_set_gf, libgbc), Cint, (Ptr{Cvoid}, Cint, Cint, Ptr{Cvoid}),
                e.h, k - 1, eltype(g) <: Complex ? 1 : 0, g))
end

function set_props!(e::GB300Ensemble, k::Integer, p::RateStateQuasiDynamicProperty)
    check(ccall((:gbc_ensemble_set_fault_props, libgbc), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble, Cdouble, Cdouble, Cdouble),
                e.h, k - 1, p.a, p.b, p.L, p.σ, p.η, p.vpl, p.f₀, p.v₀))
end

"""
    solve_gb300(e, u0s, tspans, alg; reltol, abstol, dt, dtmax, maxiters, log_theta)

Integrates model k from `tspans[k][1]` to `tspans[k][2]` starting from `u0s[k]` (an ArrayPartition
(v, θ, δ) as `assemble` takes), all models in one batched call; returns the final states
(ArrayPartitions like `u0s`) and one stats entry per model. `log_theta`: integrate ln θ in place of
θ (the state handed back is θ either way); by default for Tsit5 only, since a multistep method on
ln θ lands a tolerance-sized distance from the θ solution.
"""
function solve_gb300(e::GB300Ensemble, u0s::AbstractVector, tspans::AbstractVector, alg; reltol=1e-6, abstol=1e-8,
                     dt=1e-8, dtmax=Inf, dtmin=1e-14, maxiters::Integer=10^9, log_theta::Bool=!(alg isa VCABM5))
    n = e.nmodels
    (length(u0s) == n && length(tspans) == n) || throw(DimensionMismatch("one state and one time span per model"))
    code = alg isa VCABM5 ? Cint(1) : alg isa Tsit5 ? Cint(0) : throw(ArgumentError("VCABM5() or Tsit5()"))
    check(ccall((:gbc_ensemble_set_log_theta, libgbc), Cint, (Ptr{Cvoid}, Cint), e.h, log_theta))
    o = GbcSolverOpts(reltol, abstol, dt, isfinite(dtmax) ? dtmax : 1e300, dtmin, maxiters, code)
    offset(k) = Int(ccall((:gbc_ensemble_state_offset, libgbc), Clonglong, (Ptr{Cvoid}, Cint), e.h, k - 1))
    u = zeros(Int(ccall((:gbc_ensemble_state_len, libgbc), Clonglong, (Ptr{Cvoid},), e.h)))
    for k in 1:n
        flat = reduce(vcat, (vec(copy(x)) for x in u0s[k].x))
        copyto!(u, offset(k) + 1, flat, 1, length(flat))
    end
    t0 = Float64[ts[1] for ts in tspans]
    t1 = Float64[ts[2] for ts in tspans]
    st = Vector{GbcStatsC}(undef, n)
    rc = ccall((:gbc_ensemble_integrate, libgbc), Cint,
               (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ref{GbcSolverOpts}, Ptr{GbcStatsC}),
               e.h, u, t0, t1, o, st)
    rc == 0 || rc == -5 || check(rc)
    outs = map(1:n) do k
        out = deepcopy(u0s[k])
        off = offset(k)
        for x in out.x
            copyto!(x, 1, u, off + 1, length(x)); off += length(x)
        end
        out
    end
    return outs, st
end

end # module
