"""
    MCPhyloGPU

Julia binding of libmcphylo_gpu.so for MCPhylo.jl: `GPUPhyloDist` wraps a
`PhyloDist` and evaluates `logpdf` / `gradlogpdf` on a GB300 through `ccall`.

    using MCPhylo, MCPhyloGPU
    pd  = PhyloDist(tree, pden, [1.0], [1.0], JC)
    gpd = GPUPhyloDist(pd; precision = :f32)      # or :f64 (plain FP64), :tf32 / :bf16 / :tf32x3 (K >= 9)
    logpdf(gpd, df); gradlogpdf(gpd, df)          # same results and layouts as pd

In a model, use `GPUPhyloDist(PhyloDist(...))` where the reference uses
`PhyloDist(...)`.  The C ABI is declared in include/mcphylo_gpu.h.
"""
module MCPhyloGPU

using MCPhylo
import MCPhylo: logpdf, gradlogpdf, DiscreteMatrixDistribution, PhyloDist
using MCPhylo: post_order, get_branchlength_vector, get_leaves, get_mother

export GPUPhyloDist

const libmcphy = get(ENV, "MCPHYLO_GPU_LIB",
                     joinpath(@__DIR__, "..", "mcphylo_gb300", "libmcphylo_gpu.so"))

mutable struct Handle
    ptr::Ptr{Cvoid}
end

function check(st::Integer, h::Ptr{Cvoid})
    st == 0 && return nothing
    msg = h == C_NULL ? "status $st" :
          unsafe_string(ccall((:mcphy_last_error, libmcphy), Cstring, (Ptr{Cvoid},), h))
    st == -2 && throw(DimensionMismatch(msg))
    st in (-1, -3, -9) && throw(ArgumentError(msg))
    error("libmcphylo_gpu: $msg (status $st)")
end

const PRECISIONS = Dict(:f32 => 0, :f64 => 1, :tf32 => 2, :bf16 => 3, :tf32x3 => 4)

function Handle(nbase::Int, nrates::Int, precision::Symbol)
    haskey(PRECISIONS, precision) ||
        throw(ArgumentError("precision must be one of $(sort(collect(keys(PRECISIONS))))"))
    r = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:mcphy_create, libmcphy), Cint, (Int64, Int64, Cint, Ref{Ptr{Cvoid}}),
               nbase, nrates, PRECISIONS[precision], r)
    check(st, C_NULL)
    h = Handle(r[])
    finalizer(h) do x
        x.ptr == C_NULL || ccall((:mcphy_destroy, libmcphy), Cint, (Ptr{Cvoid},), x.ptr)
        x.ptr = C_NULL
    end
    return h
end

"""
    GPUPhyloDist(pd::PhyloDist; precision = :f64)

`pd` evaluated by the engine.  The tree, branch lengths, model and data are
re-sent only when they changed since the previous call (a sampler's leapfrog
step sends the branch lengths and reads back logL and the gradient).
"""
mutable struct GPUPhyloDist{P<:PhyloDist} <: DiscreteMatrixDistribution
    pd::P
    h::Handle
    parent::Vector{Int64}
    blen::Vector{Float64}
    data::Array{Float64,3}
end

function GPUPhyloDist(pd::PhyloDist; precision::Symbol = :f64)
    h = Handle(pd.nbase, length(pd.rates), precision)
    U, D, Uinv, mu = pd.substitution_model(pd.base_freq, pd.substitution_rates)
    check(ccall((:mcphy_set_model, libmcphy), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Float64, Ptr{Float64},
                 Ptr{Float64}),
                h.ptr, Matrix{Float64}(U), Vector{Float64}(D), Matrix{Float64}(Uinv), mu,
                pd.base_freq, pd.rates), h.ptr)
    GPUPhyloDist(pd, h, Int64[], Float64[], Array{Float64,3}(undef, 0, 0, 0))
end

Base.size(d::GPUPhyloDist) = size(d.pd)
Base.minimum(d::GPUPhyloDist) = -Inf
Base.maximum(d::GPUPhyloDist) = Inf

# parent[num] = mother's num (0 for the root), as the C ABI expects
function parent_array(tree)
    po = post_order(tree)
    parent = zeros(Int64, length(po))
    for n in po
        parent[n.num] = n.root ? 0 : get_mother(n).num
    end
    parent
end

function sync!(d::GPUPhyloDist, x::AbstractArray{<:Real,3})
    tree = d.pd.tree
    parent = parent_array(tree)
    blen = Vector{Float64}(get_branchlength_vector(tree))
    if parent != d.parent
        check(ccall((:mcphy_set_tree, libmcphy), Cint,
                    (Ptr{Cvoid}, Int64, Ptr{Int64}, Ptr{Float64}),
                    d.h.ptr, length(parent), parent, blen), d.h.ptr)
        d.parent = parent
        d.blen = blen
    elseif blen != d.blen
        check(ccall((:mcphy_set_branch_lengths, libmcphy), Cint, (Ptr{Cvoid}, Ptr{Float64}),
                    d.h.ptr, blen), d.h.ptr)
        d.blen = blen
    end
    if size(x) != size(d.data) || x != d.data
        xd = Array{Float64,3}(x)
        leaves = Int64[l.num for l in get_leaves(tree)]
        check(ccall((:mcphy_set_data, libmcphy), Cint,
                    (Ptr{Cvoid}, Ptr{Float64}, Int64, Int64, Ptr{Int64}, Int64),
                    d.h.ptr, xd, size(xd, 2), size(xd, 3), leaves, length(leaves)), d.h.ptr)
        d.data = xd
    end
    nothing
end

function logpdf(d::GPUPhyloDist, x::AbstractArray{<:Real,3})::Float64
    sync!(d, x)
    ll = Ref{Float64}(0.0)
    check(ccall((:mcphy_logpdf, libmcphy), Cint, (Ptr{Cvoid}, Ref{Float64}), d.h.ptr, ll),
          d.h.ptr)
    ll[]
end

function gradlogpdf(d::GPUPhyloDist, x::AbstractArray)
    sync!(d, x)
    ll = Ref{Float64}(0.0)
    grad = Vector{Float64}(undef, length(d.parent) - 1)
    check(ccall((:mcphy_logpdf_grad, libmcphy), Cint, (Ptr{Cvoid}, Ref{Float64}, Ptr{Float64}),
                d.h.ptr, ll, grad), d.h.ptr)
    ll[], grad
end

# ------------------------------------------------------------------ reverse mode
# `loglik(gpd, blen)`: the log-likelihood as a function of the branch-length vector
# (num order), with a ChainRules rrule whose pullback is the engine's adjoint
# gradient, so Zygote (which MCPhylo uses) differentiates through it.
import ChainRulesCore

function loglik(d::GPUPhyloDist, blen::AbstractVector{<:Real})
    check(ccall((:mcphy_set_branch_lengths, libmcphy), Cint, (Ptr{Cvoid}, Ptr{Float64}),
                d.h.ptr, Vector{Float64}(blen)), d.h.ptr)
    d.blen = Vector{Float64}(blen)
    ll = Ref{Float64}(0.0)
    check(ccall((:mcphy_logpdf, libmcphy), Cint, (Ptr{Cvoid}, Ref{Float64}), d.h.ptr, ll), d.h.ptr)
    ll[]
end

function ChainRulesCore.rrule(::typeof(loglik), d::GPUPhyloDist, blen::AbstractVector{<:Real})
    check(ccall((:mcphy_set_branch_lengths, libmcphy), Cint, (Ptr{Cvoid}, Ptr{Float64}),
                d.h.ptr, Vector{Float64}(blen)), d.h.ptr)
    d.blen = Vector{Float64}(blen)
    ll = Ref{Float64}(0.0)
    grad = Vector{Float64}(undef, length(blen))
    check(ccall((:mcphy_logpdf_grad, libmcphy), Cint, (Ptr{Cvoid}, Ref{Float64}, Ptr{Float64}),
                d.h.ptr, ll, grad), d.h.ptr)
    pullback(Δ) = (ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), Δ .* grad)
    return ll[], pullback
end

export loglik

end # module
