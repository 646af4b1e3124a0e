"""
    GaussMLEGB300

`ccall` binding of libgaussmle_sm100a.so (include/gaussmle_gb300.h) for
GaussMLE.jl.  It replaces the GPU branches of `fit` (src/interface.jl:217-263,
:334-370, :421-457): everything before them (validation, `to_pixel_units`,
corners) and after them (p-values, `create_localization_result`, `to_smld`)
stays in GaussMLE, so `fit` still returns the same `BasicSMLD` emitters.

There is no CPU fallback: `Context()` throws when the library or an sm_103a
GPU is missing.
"""
module GaussMLEGB300

using GaussMLE: GaussMLE, PSFModel, GaussianXYNB, GaussianXYNBS, GaussianXYNBSXSY,
                AstigmaticXYZNB, ParameterConstraints

const libgmle = get(ENV, "GAUSSMLE_GB300_LIB",
                    joinpath(@__DIR__, "..", "lib", "libgaussmle_sm100a.so"))

const CAMERA_POISSON = Int32(0)
const CAMERA_SCMOS = Int32(1)
const CAMERA_SCMOS_ADU = Int32(2)

# gmle_fit_desc
struct FitDesc
    model::Int32
    box::Int32
    iterations::Int32
    camera::Int32
    psf::NTuple{8,Float32}
    lower::NTuple{6,Float32}
    upper::NTuple{6,Float32}
    max_step::NTuple{6,Float32}
    method::Int32   # 0: the reference's Newton step; 1: full-Hessian (Fisher scoring, LM damping)
end

model_id(::GaussianXYNB) = Int32(0)
model_id(::GaussianXYNBS) = Int32(1)
model_id(::GaussianXYNBSXSY) = Int32(2)
model_id(::AstigmaticXYZNB) = Int32(3)

psf_vector(p::GaussianXYNB) = (Float32(p.σ), 0f0, 0f0, 0f0, 0f0, 0f0, 0f0, 0f0)
psf_vector(::GaussianXYNBS) = ntuple(_ -> 0f0, 8)
psf_vector(::GaussianXYNBSXSY) = ntuple(_ -> 0f0, 8)
psf_vector(p::AstigmaticXYZNB) = Float32.((p.σx₀, p.σy₀, p.Ax, p.Ay, p.Bx, p.By, p.γ, p.d))

pad6(v) = ntuple(k -> k <= length(v) ? Float32(v[k]) : 0f0, 6)

function FitDesc(psf_pixels::PSFModel, box::Integer, iterations::Integer, camera::Integer,
                 c::ParameterConstraints; method::Integer = 0)
    FitDesc(model_id(psf_pixels), Int32(box), Int32(iterations), Int32(camera),
            psf_vector(psf_pixels), pad6(c.lower), pad6(c.upper), pad6(c.max_step), Int32(method))
end

mutable struct Context
    ptr::Ptr{Cvoid}
end

function Context(device::Integer = 0)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:gmle_create, libgmle), Cint, (Ref{Ptr{Cvoid}}, Cint), r, device)
    st == 0 || error("GaussMLEGB300: no usable GB300 on device $device (status $st); " *
                     "this backend has no CPU fallback")
    ctx = Context(r[])
    finalizer(c -> ccall((:gmle_destroy, libgmle), Cvoid, (Ptr{Cvoid},), c.ptr), ctx)
    return ctx
end

function check(ctx::Context, st::Cint)
    st == 0 && return nothing
    msg = unsafe_string(ccall((:gmle_last_error, libgmle), Cstring, (Ptr{Cvoid},), ctx.ptr))
    error("GaussMLEGB300 (status $st): $msg")
end

const DEFAULT_CONTEXT = Ref{Union{Nothing,Context}}(nothing)
default_context() = something(DEFAULT_CONTEXT[], (DEFAULT_CONTEXT[] = Context(0)))

"""
    set_calibration!(ctx, variance, gain=nothing, offset=nothing)

Upload full-sensor (ny, nx) maps once; they stay resident on the GPU
(replaces the per-batch variance-map copy of src/interface.jl:431-432).
"""
function set_calibration!(ctx::Context, variance::AbstractMatrix, gain = nothing,
                          offset = nothing)
    v = Matrix{Float32}(variance)
    g = gain === nothing ? C_NULL : Matrix{Float32}(gain)
    o = offset === nothing ? C_NULL : Matrix{Float32}(offset)
    GC.@preserve v g o begin
        st = ccall((:gmle_set_calibration, libgmle), Cint,
                   (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Int32, Int32),
                   ctx.ptr, v, g, o, size(v, 1), size(v, 2))
    end
    check(ctx, st)
end

"""
    fit!(results, uncertainties, log_likelihoods, data, psf_pixels, camera,
         x_corners, y_corners, constraints, iterations; ctx)

The GPU branch of `fit`: `data` is (box, box, n) Float32, `results` and
`uncertainties` (P, n), `log_likelihoods` (n) - the arrays GaussMLE already
allocates (src/interface.jl:195-197).  Returns the per-ROI flags.
"""
function fit!(results::Matrix{Float32}, uncertainties::Matrix{Float32},
              log_likelihoods::Vector{Float32}, data::Array{Float32,3}, psf_pixels::PSFModel,
              camera::Integer, x_corners::Vector{Int32}, y_corners::Vector{Int32},
              constraints::ParameterConstraints, iterations::Integer;
              ctx::Context = default_context())
    box, n = size(data, 1), size(data, 3)
    desc = Ref(FitDesc(psf_pixels, box, iterations, camera, constraints))
    flags = Vector{UInt8}(undef, n)
    GC.@preserve data x_corners y_corners results uncertainties log_likelihoods flags begin
        st = ccall((:gmle_fit, libgmle), Cint,
                   (Ptr{Cvoid}, Ref{FitDesc}, Ptr{Float32}, Ptr{Int32}, Ptr{Int32}, Int64,
                    Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Ptr{UInt8}),
                   ctx.ptr, desc, data, x_corners, y_corners, n, results, uncertainties,
                   log_likelihoods, flags)
    end
    check(ctx, st)
    return flags
end

"""
    pvalues(log_likelihoods, box, nparams; ctx)

The p-value loop after the GPU branch (src/interface.jl:265-275), on the GPU:
`1 - Float32(cdf(Chisq(box^2 - nparams), -2 llr))`.
"""
function pvalues(log_likelihoods::Vector{Float32}, box::Integer, nparams::Integer;
                 ctx::Context = default_context())
    pv = Vector{Float32}(undef, length(log_likelihoods))
    GC.@preserve log_likelihoods pv begin
        st = ccall((:gmle_pvalues, libgmle), Cint,
                   (Ptr{Cvoid}, Ptr{Float32}, Int64, Int32, Ptr{Float32}),
                   ctx.ptr, log_likelihoods, length(log_likelihoods), Int32(box^2 - nparams), pv)
    end
    check(ctx, st)
    return pv
end

# ---- serving loop (gmle_server_* / gmle_submit* / gmle_wait) ------------------

# gmle_group: one request; host pointers for gmle_submit / gmle_submit_many
struct GmleGroup
    desc::FitDesc
    data::Ptr{Float32}
    x_corners::Ptr{Int32}
    y_corners::Ptr{Int32}
    n::Int64
    params::Ptr{Float32}
    crlb::Ptr{Float32}
    llr::Ptr{Float32}
    flags::Ptr{UInt8}
end

# gmle_server_config (zeros: the defaults)
struct ServerConfig
    hbm_budget_bytes::Int64
    max_inflight_steps::Int32
    max_step_rois::Int64
    max_pending::Int32
    use_graphs::Int32
end

function server_start!(ctx::Context; hbm_budget_bytes = 0, max_inflight_steps = 0,
                       max_step_rois = 0, max_pending = 0, use_graphs = false)
    cfg = Ref(ServerConfig(hbm_budget_bytes, max_inflight_steps, max_step_rois, max_pending,
                           Int32(use_graphs)))
    check(ctx, ccall((:gmle_server_start, libgmle), Cint, (Ptr{Cvoid}, Ref{ServerConfig}),
                     ctx.ptr, cfg))
end

server_stop!(ctx::Context) = check(ctx, ccall((:gmle_server_stop, libgmle), Cint,
                                              (Ptr{Cvoid},), ctx.ptr))

"""
    submit!(ctx, requests) -> tickets

Queues `requests` (a `Vector{GmleGroup}` whose host arrays the caller keeps
alive until each ticket is waited for) in one `gmle_submit_many` call.
"""
function submit!(ctx::Context, requests::Vector{GmleGroup})
    tickets = Vector{UInt64}(undef, length(requests))
    accepted = Ref{Int32}(0)
    st = ccall((:gmle_submit_many, libgmle), Cint,
               (Ptr{Cvoid}, Ptr{GmleGroup}, Int32, Ptr{UInt64}, Ref{Int32}),
               ctx.ptr, requests, Int32(length(requests)), tickets, accepted)
    check(ctx, st)
    return tickets
end

"""
    wait!(ctx, ticket; timeout_ns = -1)

Blocks until the request is done (its outputs written) or fails.
"""
wait!(ctx::Context, ticket::UInt64; timeout_ns::Integer = -1) =
    check(ctx, ccall((:gmle_wait, libgmle), Cint, (Ptr{Cvoid}, UInt64, Int64), ctx.ptr, ticket,
                     Int64(timeout_ns)))

end # module
