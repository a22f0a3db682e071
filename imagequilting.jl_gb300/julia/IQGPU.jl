# IQGPU.jl -- Julia binding of libiqgpu.so: a drop-in `iqsim` for ImageQuilting.jl users.
#
# Same signature, defaults, assertions and return types as ImageQuilting.iqsim
# (src/iqsim.jl:50-63,145,314); the tile loop runs in the CUDA library through the C ABI of
# include/iqgpu.h. Coordinates are converted from 1-based CartesianIndex to 0-based, arrays are
# passed column-major as they are. `rng` seeds the library's Philox4x32-10 streams (a UInt64
# drawn from it), which replace Julia's Xoshiro stream inside the simulation.
module IQGPU

using Random

export iqsim, voxelreuse

const LIB = Ref{String}(joinpath(@__DIR__, "..", "libiqgpu.so"))

struct SimParams
  ndim::Int32
  tilesize::NTuple{3,Int64}
  simsize::NTuple{3,Int64}
  overlap::NTuple{3,Float64}
  tol::Float64
  path::Int32
  nreal::Int32
  debug::Int32
  seed::UInt64
  real0::Int64
end

struct HardData
  n::Int64
  coords::Ptr{Int64}
  values::Ptr{Float64}
end

struct SoftData
  aux::Ptr{Float32}
  auxsize::NTuple{3,Int64}
  auxti::Ptr{Float32}
end

const PATHS = Dict(:raster => Int32(0), :dilation => Int32(1), :random => Int32(2))

lasterror() = unsafe_string(ccall((:iq_last_error, LIB[]), Cstring, ()))
check(rc) = rc == 0 || error("libiqgpu error $rc: $(lasterror())")

mutable struct Context
  h::Ptr{Cvoid}
  function Context(device::Integer=0)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:iq_ctx_create, LIB[]), Cint, (Cint, Ptr{Ptr{Cvoid}}), device, r))
    c = new(r[])
    finalizer(x -> ccall((:iq_ctx_destroy, LIB[]), Cint, (Ptr{Cvoid},), x.h), c)
    c
  end
end

# Tuning knob of a context (iq_set_option; include/iqgpu.h lists the names and ranges)
setoption!(c::Context, name::AbstractString, value::Integer) =
  check(ccall((:iq_set_option, LIB[]), Cint, (Ptr{Cvoid}, Cstring, Int64), c.h, name, value))

const DEFAULT = Ref{Union{Nothing,Context}}(nothing)
context() = (DEFAULT[] === nothing && (DEFAULT[] = Context(0)); DEFAULT[])

pad3(t, fill) = ntuple(i -> i <= length(t) ? t[i] : fill, 3)

function iqsim(trainimg::AbstractArray{T,N}, tilesize::Dims{N}, simsize::Dims{N}=size(trainimg);
               overlap::NTuple{N,<:Real}=ntuple(i -> 1 / 6, N), soft::AbstractVector=[],
               hard::Dict=Dict(), tol::Real=0.1, path::Symbol=:raster, nreal::Integer=1,
               debug::Bool=false, showprogress::Bool=true,
               rng=Random.default_rng()) where {T,N}
  @assert all(0 .< tilesize .≤ size(trainimg)) "invalid tile size"
  @assert all(simsize .≥ tilesize) "invalid grid size"
  @assert all(0 .< overlap .< 1) "overlaps must be in range (0,1)"
  @assert 0 < tol ≤ 1 "tolerance must be in range (0,1]"
  @assert path ∈ [:raster, :dilation, :random] "invalid simulation path"
  @assert nreal > 0 "invalid number of realizations"
  for (aux, auxTI) in soft
    @assert all(size(aux) .≥ simsize) "soft data size < grid size"
    @assert size(auxTI) == size(trainimg) "auxiliary TI must have the same size as TI"
  end
  if !isempty(hard)
    cs = [coord[i] for i in 1:N, coord in keys(hard)]
    @assert all(maximum(cs, dims=2) .≤ simsize) "hard data coordinates outside of grid"
    @assert all(minimum(cs, dims=2) .> 0) "hard data coordinates must be positive indices"
  end

  ctx = context()
  # training image: missing -> NaN, Float32 or Float64 as given, other types as Float64
  F = nonmissingtype(T) <: AbstractFloat ? nonmissingtype(T) : Float64
  TI = Array{F}(replace(trainimg, missing => F(NaN)))
  dtype = F === Float32 ? Int32(0) : Int32(1)
  TI64 = F === Float32 || F === Float64 ? TI : Array{Float64}(TI)
  check(ccall((:iq_set_ti, LIB[]), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int32, Int32, Ptr{Int64}),
              ctx.h, TI64, dtype, N, collect(Int64, size(TI))))

  # hard data: 0-based coordinates, one row per datum
  ks = collect(keys(hard))
  coords = Int64[ks[j][i] - 1 for i in 1:N, j in eachindex(ks)]
  vals = Float64[Float64(coalesce(hard[k], NaN)) for k in ks]
  hd = Ref(HardData(length(ks), pointer(coords), pointer(vals)))

  # soft data: Float32 copies with missing -> NaN
  softs = [(Array{Float32}(replace(a, missing => NaN32)), Array{Float32}(replace(b, missing => NaN32)))
           for (a, b) in soft]
  sd = [SoftData(pointer(a), pad3(size(a), 1), pointer(b)) for (a, b) in softs]

  seed = rand(rng, UInt64)
  p = Ref(SimParams(N, pad3(tilesize, 1), pad3(simsize, 1), pad3(Float64.(overlap), 0.5),
                    tol, PATHS[path], nreal, debug, seed, 0))
  nvox = prod(simsize)
  out = Vector{Float32}(undef, nvox * nreal)
  cuts = debug ? Vector{Float32}(undef, nvox * nreal) : Float32[]
  voxs = debug ? zeros(nreal) : Float64[]
  GC.@preserve coords vals softs sd out cuts voxs begin
    check(ccall((:iq_simulate, LIB[]), Cint,
                (Ptr{Cvoid}, Ref{SimParams}, Ref{HardData}, Int32, Ptr{SoftData}, Ptr{Float32},
                 Ptr{Float32}, Ptr{Float64}),
                ctx.h, p, hd, length(sd), isempty(sd) ? C_NULL : pointer(sd), out,
                debug ? pointer(cuts) : C_NULL, debug ? pointer(voxs) : C_NULL))
  end

  R = T <: AbstractFloat ? T : Union{Missing,nonmissingtype(T)}
  reals = Vector{Array{R,N}}()
  for r in 1:nreal
    g = reshape(out[(r - 1) * nvox + 1:r * nvox], simsize)
    if R <: AbstractFloat
      push!(reals, Array{R}(g))
    else
      push!(reals, convert(Array{R}, replace(Array{Float64}(g), NaN => missing)))
    end
  end
  debug || return reals
  boundarycuts = [Array{Float64}(reshape(cuts[(r - 1) * nvox + 1:r * nvox], simsize)) for r in 1:nreal]
  reals, boundarycuts, voxs
end

function voxelreuse(trainimg::AbstractArray{T,N}, tilesize::Dims{N};
                    overlap::NTuple{N,Float64}=ntuple(i -> 1 / 6, N), nreal::Integer=10,
                    kwargs...) where {T,N}
  ovlsize = @. ceil(Int, overlap * tilesize)
  ntiles = ntuple(i -> ovlsize[i] > 1 ? 2 : 1, N)
  simsize = @. ntiles * (tilesize - ovlsize) + ovlsize
  _, _, voxs = iqsim(trainimg, tilesize, simsize; overlap=overlap, nreal=nreal, debug=true, kwargs...)
  μ = sum(voxs) / length(voxs)
  σ = sqrt(sum((voxs .- μ) .^ 2) / max(length(voxs) - 1, 1))
  μ, σ
end

end # module
