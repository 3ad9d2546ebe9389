"""
    FlouCUDA

Drop-in GPU discretization for Flou.jl: `GPUDisc(disc)` wraps a `MultielementDisc` built by
Flou and hands its arrays to libflou_cuda (the C ABI of `include/flou_cuda.h`). Flou's own
`rhs!(dQ, Q, EquationConfig(gpudisc, equation), t)` and `timeintegrate` then run on the GPU.

Shipped as source: it is the binding a Flou maintainer adds; it mirrors the Python host
package `flou_cuda` that the repository tests.
"""
module FlouCUDA

using Flou
using Flou.FlouCommon: AbstractSpatialDiscretization, EquationConfig, HyperbolicEquation
import Flou.FlouCommon: rhs!, get_max_dt
using ChainRulesCore
using LinearAlgebra
using OrdinaryDiffEq

export GPUDisc, SSPRK3GPU, LowStorageGPU, GPUBatch, solve_functional, solve_functional_batch
export set_limiter!, monitor, record_monitors!, take_monitors!

const libflou = joinpath(@__DIR__, "..", "..", "..", "lib", "libflou_cuda.so")

# ---- C structs and status ------------------------------------------------------------------
struct FlouConfig
    dim::Int32
    equation::Int32
    gamma::Float64
    advection::NTuple{3,Float64}
    volume_op::Int32
    twopoint_flux::Int32
    numflux::Int32
    numflux_avg::Int32
    numflux_intensity::Float64
    nnodes::Int32
end

const FLOU_ERR_NONPHYSICAL = 3
const PTR_HOST = Int32(0)
const PTR_DEVICE = Int32(1)

function check(status, ctx)
    status == 0 && return nothing
    msg = ctx == C_NULL ? "" :
          unsafe_string(ccall((:flou_last_error, libflou), Cstring, (Ptr{Cvoid},), ctx))
    status == FLOU_ERR_NONPHYSICAL && throw(DomainError(msg, "non-physical state"))
    error("libflou_cuda status $status: $msg")
end

# ---- configuration from Flou's objects -------------------------------------------------------
eqcode(::LinearAdvection) = Int32(0)
eqcode(::BurgersEquation) = Int32(1)
eqcode(::EulerEquation) = Int32(2)

tpcode(::StdAverage) = Int32(0)
tpcode(::ChandrasekharAverage) = Int32(1)

nfcode(::StdAverage) = Int32(0)
nfcode(::LxF) = Int32(1)
nfcode(::ChandrasekharAverage) = Int32(2)
nfcode(::ScalarDissipation) = Int32(5)
nfcode(::MatrixDissipation) = Int32(6)

# the central flux inside LxF / ScalarDissipation / MatrixDissipation, and their intensity
has_avg(nf) = nf isa LxF || nf isa ScalarDissipation || nf isa MatrixDissipation

function flou_config(disc, equation)
    op = disc.operators[1]
    nf = op.numflux
    adv = equation isa LinearAdvection ? (Tuple(equation.a)..., zeros(3 - length(equation.a))...) : (0.0, 0.0, 0.0)
    vol = op isa HybridDivOperator ? Int32(2) : op isa SplitDivOperator ? Int32(1) : Int32(0)
    tp = (op isa SplitDivOperator || op isa HybridDivOperator) ? tpcode(op.tpflux) : Int32(0)
    avg = has_avg(nf) ? (nf.avg isa ChandrasekharAverage ? Int32(2) : Int32(0)) : Int32(0)
    inten = has_avg(nf) ? Float64(nf.intensity) : 1.0
    gamma = equation isa EulerEquation ? Float64(equation.γ) : 1.4
    return FlouConfig(Int32(spatialdim(disc)), eqcode(equation), gamma, Float64.(adv), vol, tp,
                      nfcode(nf), avg, inten, Int32(length(disc.std.basis.ξ)))
end

# ---- the drop-in discretization --------------------------------------------------------------
mutable struct GPUDisc{ND,RT,D} <: AbstractSpatialDiscretization{ND,RT}
    disc::D                 # Flou's MultielementDisc (host arrays come from it)
    ctx::Ptr{Cvoid}
end

"""
    GPUDisc(disc::MultielementDisc, equation)

Uploads the operators (StdSegment.jl:77-89), the connectivity after `apply_periodicBCs!`
(Mesh.jl:236-322), the boundary conditions and the geometry of `disc` to a libflou_cuda
context. Cartesian and UnstructuredMesh (straight-sided, per-node) geometry are accepted.
"""
function GPUDisc(disc::MultielementDisc{ND,RT}, equation) where {ND,RT}
    cfg = Ref(flou_config(disc, equation))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:flou_create, libflou), Int32, (Ref{FlouConfig}, Ref{Ptr{Cvoid}}), cfg, out)
    st == 0 || error("flou_create rejected the configuration (status $st)")
    ctx = out[]
    s = disc.std.face isa Flou.StdPoint ? disc.std : disc.std   # segment matrices are shared
    D, Ds, Dsh = Matrix{Float64}(s.D), Matrix{Float64}(s.Ds), Matrix{Float64}(s.D♯)
    ω = Vector{Float64}(disc.std.basis.ω)
    ll, lr = Vector{Float64}(s.l[1]), Vector{Float64}(s.l[2])
    gl, gr = Vector{Float64}(s.∂g[1]), Vector{Float64}(s.∂g[2])
    GC.@preserve D Ds Dsh ω ll lr gl gr check(ccall((:flou_set_operators, libflou), Int32,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}), ctx, D, Ds, Dsh, ω, ll, lr, gl, gr), ctx)
    op = disc.operators[1]
    if op isa HybridDivOperator   # subcell FV flux and blending constant (OpDivergence.jl:452-470)
        fv = op.fvflux
        fvavg = has_avg(fv) ? (fv.avg isa ChandrasekharAverage ? Int32(2) : Int32(0)) : Int32(0)
        fvint = has_avg(fv) ? Float64(fv.intensity) : 1.0
        check(ccall((:flou_set_hybrid, libflou), Int32, (Ptr{Cvoid}, Int32, Int32, Float64, Float64),
                    ctx, nfcode(fv), fvavg, fvint, Float64(op.blend)), ctx)
    end
    mesh = disc.mesh
    ne, nf = nelements(mesh), nfaces(mesh)
    faceinds = Int32.(mesh.elements.faceinds)
    facepos = Int32.(mesh.elements.facepos)
    eleminds = Int32.(mesh.faces.eleminds)
    elempos = Int32.(mesh.faces.elempos)
    orient = UInt8.(mesh.faces.orientation)
    bdidx = zeros(Int32, nf)
    for ib in eachboundary(mesh), f in eachbdface(mesh, ib)
        bdidx[f] = ib
    end
    GC.@preserve faceinds facepos eleminds elempos orient bdidx check(ccall((:flou_set_mesh, libflou), Int32,
        (Ptr{Cvoid}, Int32, Int32, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{UInt8}, Ptr{Int32}),
        ctx, ne, nf, faceinds, facepos, eleminds, elempos, orient, bdidx), ctx)
    kinds = Int32[bc isa EulerSlipBC ? 3 : (bc isa EulerInflowBC || bc isa GenericBC) ? 2 : 1 for bc in disc.bcs]
    states = zeros(Float64, 5, length(kinds))
    nfd = length(disc.std.basis.ξ)^(ND - 1)
    field = nothing   # flou_set_bc_field's states, 5 per face node, face by face
    for (i, bc) in enumerate(disc.bcs)
        bc isa EulerInflowBC && (states[1:length(bc.Qext), i] .= bc.Qext)
        if bc isa GenericBC   # FlouSpatial.jl:80-91
            q = genericbc_state(bc, disc, i, equation)
            if q isa Vector   # one external state on the whole boundary: an inflow state
                states[1:length(q), i] .= q
            else              # a state per face node: FLOU_BC_STATE_FIELD
                kinds[i] = 4
                field === nothing && (field = zeros(Float64, 5, nfd * nf))
                for (f, M) in q
                    field[1:size(M, 1), (f - 1) * nfd + 1:f * nfd] .= M
                end
            end
        end
    end
    GC.@preserve kinds states check(ccall((:flou_set_bcs, libflou), Int32,
        (Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{Float64}), ctx, length(kinds), kinds, states), ctx)
    if field !== nothing
        GC.@preserve field check(ccall((:flou_set_bc_field, libflou), Int32, (Ptr{Cvoid}, Ptr{Float64}),
                                       ctx, field), ctx)
    end
    g = disc.geometry
    J = Vector{Float64}(g.elements.jac)
    Ja = reduce(vcat, (vec(Matrix(M)) for M in g.elements.metric))
    frames = reduce(vcat, ([f.n..., zeros(3 - ND)..., f.t..., zeros(3 - ND)..., f.b..., zeros(3 - ND)...]
                           for f in g.faces.frames))
    fJ = Vector{Float64}(g.faces.jac)
    GC.@preserve J Ja frames fJ check(ccall((:flou_set_geometry, libflou), Int32,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}), ctx, J, Ja, frames, fJ), ctx)
    needs_subgrid = op isa HybridDivOperator || (op isa SplitDivOperator && !Flou.hasboundaries(disc.std.basis))
    if needs_subgrid && !(mesh isa CartesianMesh)
        # subcell-interface geometry (geometry.subgrids, PhysicalRegions.jl:180-300) in the layout of
        # flou_set_subgrid: element, direction, line (tpdofs_subgrid order), interface
        n = length(disc.std.basis.ξ)
        sfr = zeros(Float64, 9, n + 1, nfd, ND, ne)
        sjac = zeros(Float64, n + 1, nfd, ND, ne)
        for ie in 1:ne, d in 1:ND
            sg = g.subgrids[ie]
            for (m, sinds) in enumerate(Flou.tpdofs_subgrid(disc.std, Val(d))), (s, is) in enumerate(sinds)
                f = sg.frames[d][is]
                sfr[1:ND, s, m, d, ie] .= f.n
                sfr[4:3+ND, s, m, d, ie] .= f.t
                ND == 3 && (sfr[7:9, s, m, d, ie] .= f.b)
                sjac[s, m, d, ie] = sg.jac[d][is]
            end
        end
        GC.@preserve sfr sjac check(ccall((:flou_set_subgrid, libflou), Int32,
            (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), ctx, sfr, sjac), ctx)
    end
    gd = GPUDisc{ND,RT,typeof(disc)}(disc, ctx)
    finalizer(x -> ccall((:flou_destroy, libflou), Int32, (Ptr{Cvoid},), x.ctx), gd)
    return gd
end

# rhs!(dQ, Q, p, t): Flou's residual on the GPU (Hyperbolic.jl:31-69).
function rhs!(dQ::Matrix{Float64}, Q::Matrix{Float64}, p::EquationConfig{<:GPUDisc}, t::Real)
    ctx = p.disc.ctx
    GC.@preserve dQ Q check(ccall((:flou_rhs, libflou), Int32,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Float64, Int32), ctx, dQ, Q, t, PTR_HOST), ctx)
    return nothing
end

function get_max_dt(q::Matrix{Float64}, disc::GPUDisc, ::Any, cfl)
    dt = Ref{Float64}(0.0)
    GC.@preserve q check(ccall((:flou_max_dt, libflou), Int32,
        (Ptr{Cvoid}, Ptr{Float64}, Float64, Ref{Float64}, Int32), disc.ctx, q, cfl, dt, PTR_HOST), disc.ctx)
    return dt[]
end

"""
The external state of a GenericBC evaluated at every face node of boundary `ib`
(`Qext(nothing, x, nothing, 0, equation)`: a state given by the position alone).  Returns one
vector when every node gets the same state, else `face => (nvars x face nodes)` pairs in the
face-dof order of `geometry.faces.coords`.
"""
function genericbc_state(bc, disc, ib, equation)
    per_face = [f => reduce(hcat, [Vector{Float64}(bc.Qext(nothing, x, nothing, 0.0, equation))
                                   for x in disc.geometry.faces.coords[f]])
                for f in eachbdface(disc.mesh, ib)]
    q1 = per_face[1].second[:, 1]
    all(p -> all(==(q1), eachcol(p.second)), per_face) && return q1
    return per_face
end

"SSP-RK3 run entirely on the GPU (one CUDA graph per step)."
struct SSPRK3GPU end

"""
    LowStorageGPU(solver)

A 2N-storage method of OrdinaryDiffEq (ORK256, CarpenterKennedy2N54, ...: the LowStorageRK2N
family) run on the GPU by `flou_step` after `flou_set_integrator`; its coefficients come from
OrdinaryDiffEq's own tableau (`<Name>ConstantCache(Float64, Float64)`: A2end, B1, B2end).  The
stage limiter of the solver is not carried over: set it with `set_limiter!`.
"""
struct LowStorageGPU
    A::Vector{Float64}
    B::Vector{Float64}
end

function LowStorageGPU(solver)
    cache = getproperty(OrdinaryDiffEq, Symbol(nameof(typeof(solver)), "ConstantCache"))
    tab = cache(Float64, Float64)
    return LowStorageGPU(vcat(0.0, collect(tab.A2end)), vcat(tab.B1, collect(tab.B2end)))
end

# runs f() with the context stepping by `integrator` (SSP-RK3 again afterwards)
with_integrator(f, disc::GPUDisc, ::SSPRK3GPU) = f()
function with_integrator(f, disc::GPUDisc, solver::LowStorageGPU)
    A, B = solver.A, solver.B
    GC.@preserve A B check(ccall((:flou_set_integrator, libflou), Int32,
        (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}), disc.ctx, length(B), A, B), disc.ctx)
    try
        return f()
    finally
        ccall((:flou_set_integrator, libflou), Int32, (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}),
              disc.ctx, 0, C_NULL, C_NULL)
    end
end

function Flou.timeintegrate(Q0::Matrix{Float64}, disc::GPUDisc, equation, solver::LowStorageGPU, tfinal; dt,
                            kwargs...)
    return with_integrator(disc, solver) do
        Flou.timeintegrate(Q0, disc, equation, SSPRK3GPU(), tfinal; dt=dt, kwargs...)
    end
end

"""
    timeintegrate(Q0, disc::GPUDisc, equation, ::SSPRK3GPU, tfinal; dt, cfl=nothing, dtmax=Inf)

Same contract as Flou's `timeintegrate` (FlouTime.jl:34-54): returns `(sol, exetime)`, logs
"Simulation crashed!" on a DomainError.  With `cfl` the step follows
`get_cfl_callback(cfl, dtmax)` (FlouTime.jl:92-105), computed on the device by `flou_step_cfl`.
"""
function Flou.timeintegrate(Q0::Matrix{Float64}, disc::GPUDisc, equation, ::SSPRK3GPU, tfinal; dt=nothing,
                            cfl=nothing, dtmax=Inf, maxiters=10^6, kwargs...)
    Q = copy(Q0)
    t = Ref{Float64}(0.0)
    exetime = @elapsed begin
        try
            if cfl === nothing
                nsteps = round(Int, tfinal / dt)
                GC.@preserve Q check(ccall((:flou_step, libflou), Int32,
                    (Ptr{Cvoid}, Ptr{Float64}, Float64, Float64, Int32, Int32), disc.ctx, Q, dt, 0.0, nsteps,
                    PTR_HOST), disc.ctx)
                t[] = tfinal
            else
                n = Ref{Int64}(0)
                GC.@preserve Q check(ccall((:flou_step_cfl, libflou), Int32,
                    (Ptr{Cvoid}, Ptr{Float64}, Float64, Float64, Float64, Float64, Int64, Int32, Ref{Int64},
                     Ref{Float64}), disc.ctx, Q, 0.0, tfinal, cfl, dtmax, maxiters, PTR_HOST, n, t), disc.ctx)
            end
        catch e
            e isa DomainError ? (@error "Simulation crashed!") : rethrow()
        end
    end
    return ((t=[0.0, t[]], u=[Q0, Q]), exetime)
end

# ---- differentiable terminal functional --------------------------------------------------------
"""
    solve_functional(disc, Q0, c, dt, nsteps, ρtarget, w) -> J

J = 1/2 Σ w (ρ(T) - ρt)² after `nsteps` steps with per-element dissipation scales `c` (LxF
interface fluxes), or `c = nothing` for HLL, HLLC and the Scalar/MatrixDissipation fluxes, which
take no per-element scale.  The keyword `integrator` (SSPRK3GPU() or a LowStorageGPU method)
selects the time stepping that is differentiated.
Differentiable through the `rrule`s below (discrete adjoint, binomial checkpointing).
Arrays are device pointers wrapped by the caller's GPU array package (e.g. CuArray).
"""
function solve_functional end

function ChainRulesCore.rrule(::typeof(solve_functional), disc::GPUDisc, Q0, c, dt, nsteps, ρt, w; nsnap=20,
                              integrator=SSPRK3GPU())
    J = Ref{Float64}(0.0)
    g = similar(Q0)
    gc = similar(c)
    nf = Ref{Int64}(0)
    check(ccall((:flou_set_dissipation, libflou), Int32, (Ptr{Cvoid}, Ptr{Float64}, Int32), disc.ctx, pointer(c),
                PTR_DEVICE), disc.ctx)
    with_integrator(disc, integrator) do
        check(ccall((:flou_adjoint_solve, libflou), Int32,
            (Ptr{Cvoid}, Ptr{Float64}, Float64, Int32, Int32, Ptr{Float64}, Ptr{Float64}, Ref{Float64}, Ptr{Float64},
             Ptr{Float64}, Ref{Int64}),
            disc.ctx, pointer(Q0), dt, nsteps, nsnap, pointer(ρt), pointer(w), J, pointer(g), pointer(gc), nf),
            disc.ctx)
    end
    pullback(J̄) = (NoTangent(), NoTangent(), J̄ .* g, J̄ .* gc, NoTangent(), NoTangent(), NoTangent(), NoTangent())
    return J[], pullback
end

# HLL, HLLC, Scalar/MatrixDissipation: no per-element scale, so no dJ/dc (the C ABI takes a null dJdc)
function ChainRulesCore.rrule(::typeof(solve_functional), disc::GPUDisc, Q0, ::Nothing, dt, nsteps, ρt, w; nsnap=20,
                              integrator=SSPRK3GPU())
    J = Ref{Float64}(0.0)
    g = similar(Q0)
    nf = Ref{Int64}(0)
    with_integrator(disc, integrator) do
        check(ccall((:flou_adjoint_solve, libflou), Int32,
            (Ptr{Cvoid}, Ptr{Float64}, Float64, Int32, Int32, Ptr{Float64}, Ptr{Float64}, Ref{Float64}, Ptr{Float64},
             Ptr{Float64}, Ref{Int64}),
            disc.ctx, pointer(Q0), dt, nsteps, nsnap, pointer(ρt), pointer(w), J, pointer(g), C_NULL, nf), disc.ctx)
    end
    pullback(J̄) = (NoTangent(), NoTangent(), J̄ .* g, NoTangent(), NoTangent(), NoTangent(), NoTangent(), NoTangent())
    return J[], pullback
end

# ---- stage limiter and monitors (Euler.jl:541-654, FlouTime.jl:107-148) ------------------------------
"""
    set_limiter!(disc::GPUDisc, :zhang_shu, minval)

The Zhang-Shu limiter that `get_limiter_callback(disc, eq, :zhang_shu, minval)` passes to
OrdinaryDiffEq as `stage_limiter!`; here it runs after every stage inside `flou_step`'s graph.
`set_limiter!(disc, :none)` turns it off.
"""
function set_limiter!(disc::GPUDisc, name::Symbol, minval=0.0)
    kind = name == :zhang_shu ? Int32(1) : name == :none ? Int32(0) : error("Unknown limiter '$(name)'.")
    check(ccall((:flou_set_limiter, libflou), Int32, (Ptr{Cvoid}, Int32, Float64), disc.ctx, kind, minval), disc.ctx)
end

monitor_code(name::Symbol) = name in (:energy, :kinetic_energy) ? Int32(1) :
                             name == :entropy ? Int32(2) : error("Unknown monitor '$(name)'.")

"""
    monitor(disc::GPUDisc, Q::Matrix{Float64}, name) -> value

`get_monitor(disc, equation, name)` evaluated on the GPU: `:energy` / `:kinetic_energy` or `:entropy`.
"""
function monitor(disc::GPUDisc, Q::Matrix{Float64}, name::Symbol)
    v = Ref{Float64}(0.0)
    GC.@preserve Q check(ccall((:flou_monitor, libflou), Int32, (Ptr{Cvoid}, Ptr{Float64}, Int32, Ref{Float64}, Int32),
                               disc.ctx, Q, monitor_code(name), v, PTR_HOST), disc.ctx)
    return v[]
end

"""
    record_monitors!(disc, names, capacity); take_monitors!(disc) -> Matrix (nsteps × 2)

Monitors recorded after every step of `flou_step` (get_monitor_callback with iter=true) without a
host round trip; columns: kinetic energy, entropy.
"""
function record_monitors!(disc::GPUDisc, names, capacity)
    mask = reduce(|, (monitor_code(n) for n in names); init=Int32(0))
    check(ccall((:flou_set_monitors, libflou), Int32, (Ptr{Cvoid}, Int32, Int32), disc.ctx, mask, capacity), disc.ctx)
end

function take_monitors!(disc::GPUDisc, max_steps=1 << 16)
    out = zeros(2, max_steps)
    n = Ref{Int32}(0)
    check(ccall((:flou_take_monitors, libflou), Int32, (Ptr{Cvoid}, Ptr{Float64}, Int32, Ref{Int32}),
                disc.ctx, out, max_steps, n), disc.ctx)
    return permutedims(out[:, 1:n[]])
end

# ---- batched mode --------------------------------------------------------------------------------
mutable struct GPUBatch
    h::Ptr{Cvoid}
    discs::Vector{GPUDisc}
end

function GPUBatch(discs::Vector{<:GPUDisc}, states, dts::Vector{Float64})
    ctxs = [d.ctx for d in discs]
    out = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:flou_batch_create, libflou), Int32, (Int32, Ptr{Ptr{Cvoid}}, Ref{Ptr{Cvoid}}), length(ctxs), ctxs, out)
    st == 0 || error("flou_batch_create failed ($st)")
    ptrs = [pointer(q) for q in states]
    ccall((:flou_batch_set_states, libflou), Int32, (Ptr{Cvoid}, Ptr{Ptr{Float64}}, Ptr{Float64}), out[], ptrs, dts)
    b = GPUBatch(out[], discs)
    finalizer(x -> ccall((:flou_batch_destroy, libflou), Int32, (Ptr{Cvoid},), x.h), b)
    return b
end

step!(b::GPUBatch, nsteps) = ccall((:flou_batch_step, libflou), Int32, (Ptr{Cvoid}, Int32), b.h, nsteps)

"""
    solve_functional_batch(discs, Q0s, dts, nsteps, ρts, ws, budget_bytes; nstreams=8)
        -> (J, dJdQ0s, dJdcs, recomputed_steps, snapshots)

Gradients of J_k = 1/2 Σ w (ρ(T) - ρt)² for every instance in one lockstep reverse sweep under one
device-memory budget (`flou_adjoint_solve_batch`).  Arrays are device arrays of the caller's GPU
array package; each instance's dissipation scales are those set on its context.
"""
function solve_functional_batch(discs::Vector{<:GPUDisc}, Q0s, dts::Vector{Float64}, nsteps, ρts, ws,
                                budget_bytes; nstreams=8)
    n = length(discs)
    J = zeros(n)
    gs = [similar(q) for q in Q0s]
    gcs = [similar(q, d.disc.mesh.nelements) for (q, d) in zip(Q0s, discs)]
    fwd = Ref{Int64}(0)
    ns = Ref{Int32}(0)
    ptrs(v) = [pointer(x) for x in v]
    check(ccall((:flou_adjoint_solve_batch, libflou), Int32,
        (Int32, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Float64}}, Ptr{Float64}, Int32, Int64, Int32, Ptr{Ptr{Float64}},
         Ptr{Ptr{Float64}}, Ptr{Float64}, Ptr{Ptr{Float64}}, Ptr{Ptr{Float64}}, Ref{Int64}, Ref{Int32}),
        n, [d.ctx for d in discs], ptrs(Q0s), dts, nsteps, budget_bytes, nstreams, ptrs(ρts), ptrs(ws), J,
        ptrs(gs), ptrs(gcs), fwd, ns), discs[1].ctx)
    return J, gs, gcs, fwd[], ns[]
end

end # module
