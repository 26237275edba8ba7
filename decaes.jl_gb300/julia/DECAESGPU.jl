"""
    DECAESGPU

Drop-in GPU backend for DECAES.jl's voxelwise T2 path.  `T2mapSEcorr` and
`T2partSEcorr` accept DECAES's own `T2mapOptions` / `T2partOptions` and return
the same `(maps::Dict{String,Any}, dist::Array{T,4})` / `Dict{String,Any}` as
the reference (src/T2mapSEcorr.jl:148-196, src/T2partSEcorr.jl:40-71), computed
by libdecaes_gpu.so through its C ABI (include/decaes_gpu.h).

Julia is not available in the environment this library was built in, so this
module is not exercised by the test suite; the same ABI is exercised from
Python ctypes (decaes_gb300/_lib.py) and C.
"""
module DECAESGPU

using DECAES: DECAES, T2mapOptions, T2partOptions

const libdecaes = get(ENV, "DECAES_GPU_LIB", joinpath(@__DIR__, "..", "lib", "libdecaes_gpu.so"))

const REG = Dict("none" => 0, "lcurve" => 1, "gcv" => 2, "chi2" => 3, "mdp" => 4)
nan_or(x) = x === nothing ? NaN : Float64(x)

# decaes_t2map_opts
struct CT2mapOpts
    MatrixSize::NTuple{3, Int32}
    nTE::Int32
    TE::Float64
    nT2::Int32
    T2Range::NTuple{2, Float64}
    T1::Float64
    Threshold::Float64
    MinRefAngle::Float64
    nRefAngles::Int32
    nRefAnglesMin::Int32
    Reg::Int32
    Chi2Factor::Float64
    NoiseLevel::Float64
    RefConAngle::Float64
    SetFlipAngle::Float64
    SaveResidualNorm::Int32
    SaveDecayCurve::Int32
    SaveRegParam::Int32
    SaveNNLSBasis::Int32
    legacy::Int32
    precision::Int32
end
CT2mapOpts(o::T2mapOptions; precision::Symbol = :fp64) = CT2mapOpts(
    Int32.(o.MatrixSize), o.nTE, o.TE, o.nT2, Float64.(o.T2Range), o.T1, o.Threshold, o.MinRefAngle, o.nRefAngles,
    o.nRefAnglesMin, REG[o.Reg], nan_or(o.Chi2Factor), nan_or(o.NoiseLevel), o.RefConAngle, nan_or(o.SetFlipAngle),
    o.SaveResidualNorm, o.SaveDecayCurve, o.SaveRegParam, o.SaveNNLSBasis, o.legacy,
    precision === :mixed ? 1 : precision === :mixed_tc ? 2 : 0)

# decaes_t2map_out (16 pointers)
struct CT2mapOut
    p::NTuple{16, Ptr{Cvoid}}
end

# decaes_t2part_opts / decaes_t2part_out
struct CT2partOpts
    MatrixSize::NTuple{3, Int32}
    nT2::Int32
    T2Range::NTuple{2, Float64}
    SPWin::NTuple{2, Float64}
    MPWin::NTuple{2, Float64}
    Sigmoid::Float64
    legacy::Int32
end
CT2partOpts(o::T2partOptions) = CT2partOpts(Int32.(o.MatrixSize), o.nT2, Float64.(o.T2Range), Float64.(o.SPWin),
                                            Float64.(o.MPWin), nan_or(o.Sigmoid), o.legacy)
struct CT2partOut
    p::NTuple{4, Ptr{Cvoid}}
end

const CTX = Ref{Ptr{Cvoid}}(C_NULL)
function context(device::Integer = 0)
    if CTX[] == C_NULL
        CTX[] = ccall((:decaes_create, libdecaes), Ptr{Cvoid}, (Cint, Csize_t), device, 0)
        CTX[] == C_NULL && error("decaes_create failed (no usable CUDA device?)")
        atexit(() -> ccall((:decaes_destroy, libdecaes), Cvoid, (Ptr{Cvoid},), CTX[]))
    end
    return CTX[]
end

function check(rc::Cint)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:decaes_last_error, libdecaes), Cstring, (Ptr{Cvoid},), context()))
    rc == 1 ? throw(AssertionError(msg)) : error("libdecaes_gpu error $rc: $msg")
end

dtype(::Type{Float32}) = Cint(0)
dtype(::Type{Float64}) = Cint(1)
ptr(x) = x === nothing ? C_NULL : Ptr{Cvoid}(pointer(x))

"""
    T2mapSEcorr(image::Array{T,4}, opts::T2mapOptions{T}; B1map = nothing, precision = :fp64)

GPU counterpart of `DECAES.T2mapSEcorr`: same options, same outputs.
A Float32 `image` is widened to Float64 on the GPU and computed in Float64
(`precision = :fp64`, the default) or with the mixed method (`:mixed`,
`:mixed_tc`), and the results are returned as Float32 -- where DECAES.jl's own
`T2mapSEcorr(::Array{Float32,4})` computes in Float32.  Pass Float64 for
results equal to DECAES.jl's Float64 path.
"""
function T2mapSEcorr(image::Array{T, 4}, opts::T2mapOptions{T}; B1map = nothing, precision::Symbol = :fp64) where {T <: Union{Float32, Float64}}
    @assert size(image) == (opts.MatrixSize..., opts.nTE)
    fixed = opts.SetFlipAngle !== nothing
    nang = fixed ? 1 : opts.nRefAngles
    nanfill(sz...) = fill(T(NaN), sz...)
    maps = Dict{String, Any}(
        "echotimes" => zeros(T, opts.nTE), "t2times" => zeros(T, opts.nT2),
        "refangleset" => zeros(T, nang),
        "decaybasisset" => fixed ? zeros(T, opts.nTE, opts.nT2) : zeros(T, opts.nTE, opts.nT2, nang),
        (k => nanfill(opts.MatrixSize...) for k in ("gdn", "ggm", "gva", "fnr", "snr", "alpha"))...,
    )
    opts.SaveResidualNorm && (maps["resnorm"] = nanfill(opts.MatrixSize...))
    opts.SaveDecayCurve && (maps["decaycurve"] = nanfill(opts.MatrixSize..., opts.nTE))
    if opts.SaveRegParam
        maps["mu"] = nanfill(opts.MatrixSize...)
        maps["chi2factor"] = nanfill(opts.MatrixSize...)
    end
    opts.SaveNNLSBasis && (maps["decaybasis"] = fixed ? zeros(T, opts.nTE, opts.nT2) : nanfill(opts.MatrixSize..., opts.nTE, opts.nT2))
    dist = nanfill(opts.MatrixSize..., opts.nT2)
    g(k) = ptr(get(maps, k, nothing))
    out = Ref(CT2mapOut((ptr(dist), g("gdn"), g("ggm"), g("gva"), g("fnr"), g("snr"), g("alpha"), g("resnorm"),
                         g("decaycurve"), g("mu"), g("chi2factor"), g("decaybasis"), g("echotimes"), g("t2times"),
                         g("refangleset"), g("decaybasisset"))))
    copts = Ref(CT2mapOpts(opts; precision))
    b1 = B1map === nothing ? nothing : convert(Array{T, 3}, B1map)
    GC.@preserve maps dist image b1 begin
        check(ccall((:decaes_t2map, libdecaes), Cint,
                    (Ptr{Cvoid}, Ref{CT2mapOpts}, Ptr{Cvoid}, Cint, Ptr{Cvoid}, Ref{CT2mapOut}),
                    context(), copts, image, dtype(T), ptr(b1), out))
    end
    fixed && (maps["refangleset"] = maps["refangleset"][1])
    return maps, dist
end
T2mapSEcorr(image::Array{T, 4}; kwargs...) where {T} = T2mapSEcorr(image, T2mapOptions(image; kwargs...))

"""
    T2partSEcorr(dist::Array{T,4}, opts::T2partOptions{T})

GPU counterpart of `DECAES.T2partSEcorr`.
"""
function T2partSEcorr(dist::Array{T, 4}, opts::T2partOptions{T}) where {T <: Union{Float32, Float64}}
    @assert size(dist) == (opts.MatrixSize..., opts.nT2)
    maps = Dict{String, Any}(k => fill(T(NaN), opts.MatrixSize...) for k in ("sfr", "sgm", "mfr", "mgm"))
    out = Ref(CT2partOut((ptr(maps["sfr"]), ptr(maps["sgm"]), ptr(maps["mfr"]), ptr(maps["mgm"]))))
    GC.@preserve maps dist begin
        check(ccall((:decaes_t2part, libdecaes), Cint, (Ptr{Cvoid}, Ref{CT2partOpts}, Ptr{Cvoid}, Cint, Ref{CT2partOut}),
                    context(), Ref(CT2partOpts(opts)), dist, dtype(T), out))
    end
    return maps
end
T2partSEcorr(dist::Array{T, 4}; kwargs...) where {T} = T2partSEcorr(dist, T2partOptions(dist; kwargs...))

end # module
