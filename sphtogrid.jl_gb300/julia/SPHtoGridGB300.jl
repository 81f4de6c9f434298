"""
    SPHtoGridGB300

Julia binding of libsphgrid.so (include/sphgrid.h): a drop-in `sphMapping`
with the signature of SPHtoGrid.jl (src/cic_interpolation/cic_interpolation.jl:35-48)
that maps on a GB300 GPU through `ccall`.

    using SPHtoGrid, SPHKernels, SPHtoGridGB300
    par = mappingParameters(x_lim=[0.0,1.0], y_lim=[0.0,1.0], z_lim=[0.0,1.0], Npixels=256)
    img = SPHtoGridGB300.sphMapping(pos, hsml, m, rho, rho, rho; param=par, kernel=Cubic(2))

The result has the reference's layout and type (`Array{Float64,3}`), `Pos` is
centred in place as in the reference, and `precision = :fp32c` selects the
FP32-compensated deposition.
"""
module SPHtoGridGB300

using SPHtoGrid: SPHtoGrid, mappingParameters
using SPHKernels: AbstractSPHKernel, Cubic, Quintic, WendlandC4, WendlandC6, WendlandC8
using Rotations: RotXYZ  # a dependency of the reference (rotate_particles.jl)

const libsphgrid = get(ENV, "SPHGRID_LIB", joinpath(@__DIR__, "..", "libsphgrid.so"))

struct SphgParams
    x_lim::NTuple{2,Float64}
    y_lim::NTuple{2,Float64}
    z_lim::NTuple{2,Float64}
    center::NTuple{3,Float64}
    halfsize::NTuple{3,Float64}
    len2pix::Float64
    pixelSideLength::Float64
    Npixels::NTuple{3,Int64}
    boxsize::Float64
    periodic::Int32
    pad_::Int32
end

SphgParams(p::mappingParameters) = SphgParams(
    (Float64(p.x_lim[1]), Float64(p.x_lim[2])), (Float64(p.y_lim[1]), Float64(p.y_lim[2])),
    (Float64(p.z_lim[1]), Float64(p.z_lim[2])),
    (Float64(p.center[1]), Float64(p.center[2]), Float64(p.center[3])),
    (Float64(p.halfsize[1]), Float64(p.halfsize[2]), Float64(p.halfsize[3])),
    Float64(p.len2pix), Float64(p.pixelSideLength),
    (Int64(p.Npixels[1]), Int64(p.Npixels[2]), Int64(p.Npixels[3])),
    Float64(p.boxsize), Int32(p.periodic), Int32(0))

struct SphgParticles
    n::Int64
    pos_dtype::Int32
    attr_dtype::Int32
    pos::Ptr{Cvoid}
    pos_stride_p::Int64
    pos_stride_c::Int64
    hsml::Ptr{Cvoid}
    mass::Ptr{Cvoid}
    rho::Ptr{Cvoid}
    weights::Ptr{Cvoid}
    bin_q::Ptr{Cvoid}
    n_q::Int32
    pad_::Int32
    q_stride_p::Int64
    q_stride_k::Int64
end

struct SphgOptions
    dimensions::Int32
    kernel::Int32
    kernel_dim::Int32
    reduce_image::Int32
    return_both_maps::Int32
    calc_mean::Int32
    precision::Int32
    deterministic::Int32
    center::Int32
    filter::Int32
    memspace::Int32
    profile::Int32
    raw_accumulator::Int32
    reserved::NTuple{3,Int32}
end

mutable struct SphgStats
    n_in::Int64
    n_mapped::Int64
    deposits::Int64
    grid_mass::Float64
    particle_mass::Float64
    centred::SphgParams
    n_launches::Int32
    n_reruns::Int32
    phase_ms::NTuple{4,Float32}
    SphgStats() = new()
end

kernel_id(::Cubic) = 0
kernel_id(::Quintic) = 1
kernel_id(::WendlandC4) = 2
kernel_id(::WendlandC6) = 3
kernel_id(::WendlandC8) = 4

dtype_id(::Type{Float32}) = Int32(0)
dtype_id(::Type{Float64}) = Int32(1)

const CTX = Ref{Ptr{Cvoid}}(C_NULL)

function context()
    if CTX[] == C_NULL
        h = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:sphg_context_create, libsphgrid), Cint, (Cint, Ref{Ptr{Cvoid}}), 0, h)
        st == 0 || error(unsafe_string(ccall((:sphg_last_error, libsphgrid), Cstring, (Ptr{Cvoid},), C_NULL)))
        CTX[] = h[]
        atexit(() -> ccall((:sphg_context_destroy, libsphgrid), Cint, (Ptr{Cvoid},), CTX[]))
    end
    return CTX[]
end

# Particles already centred and selected (sort_z): mapped with no further
# centring or filtering (SPHG_CENTER_NONE, filter 0).
function map_selected(pos, HSML, M, Rho, Bin_Quant, Weights, par_c, kernel, show_progress, reduce_image,
                      return_both_maps, dimensions, calc_mean, precision)
    T = (eltype(HSML) == Float32 && eltype(M) == Float32 && eltype(Rho) == Float32 &&
         eltype(Bin_Quant) == Float32 && eltype(Weights) == Float32) ? Float32 : Float64
    pos = eltype(pos) <: Union{Float32,Float64} ? pos : Float64.(pos)
    hsml, m, rho, w, q = T.(HSML), T.(M), T.(Rho), T.(Weights), T.(Bin_Quant)
    N = length(m)
    nq = ndims(q) == 1 ? 1 : size(q, 1)
    P = par_c.Npixels[1]
    out = return_both_maps && dimensions == 2 ? zeros(Float64, P * P, nq + 1) :
          dimensions == 2 ? zeros(Float64, P, P, nq) : zeros(Float64, P, P, P)
    st = SphgStats()
    GC.@preserve pos hsml m rho w q out begin
        pt = SphgParticles(N, dtype_id(eltype(pos)), dtype_id(T), pointer(pos), 3, 1,
                           pointer(hsml), pointer(m), pointer(rho), pointer(w), pointer(q),
                           Int32(nq), Int32(0), ndims(q) == 1 ? 1 : nq, ndims(q) == 1 ? 0 : 1)
        kdim = hasfield(typeof(kernel), :dim) ? Int32(kernel.dim) : Int32(3)
        opt = SphgOptions(dimensions, kernel_id(kernel), kdim, reduce_image, return_both_maps,
                          calc_mean, precision === :fp32c ? 1 : 0, 0, 0, 0, 1, 0, 0, (0, 0, 0))
        status = ccall((:sphg_map, libsphgrid), Cint,
                       (Ptr{Cvoid}, Ref{SphgParams}, Ref{SphgOptions}, Ref{SphgParticles},
                        Ptr{Float64}, Ptr{Cvoid}, Ref{SphgStats}),
                       context(), SphgParams(par_c), opt, pt, pointer(out), C_NULL, st)
        status == 0 || error(unsafe_string(ccall((:sphg_last_error, libsphgrid), Cstring,
                                                 (Ptr{Cvoid},), context())))
    end
    show_progress && @info "Particles in image: $(st.n_mapped) / $N, deposits: $(st.deposits)"
    return out
end

"""
    sphMapping(Pos, HSML, M, Rho, Bin_Quant, Weights=Rho, RM=nothing;
               param, kernel, show_progress=true, parallel=false, reduce_image=true,
               return_both_maps=false, dimensions=2, calc_mean=false, stokes=false,
               sort_z=false, precision=:fp64)

The reference's `sphMapping` on the GPU.  `parallel` is ignored (one GPU);
`RM`/`stokes` (Faraday rotation) are not supported here.  With `sort_z` the
selection is the reference's own host glue (`center_particles` on the
caller's array, then `filter_particles_in_image(..., true)`: the z-sorted
index list taken at the input-order in-image mask, filter_shift.jl:6-64),
and the gathered particles are mapped on the GPU without further centring
or filtering.
"""
function sphMapping(Pos::Array{<:Real}, HSML::Array{<:Real}, M::Array{<:Real},
                    Rho::Array{<:Real}, Bin_Quant::Array{<:Real},
                    Weights::Array{<:Real}=Rho, RM=nothing;
                    param::mappingParameters, kernel::AbstractSPHKernel,
                    show_progress::Bool=true, parallel::Bool=false,
                    reduce_image::Bool=true, return_both_maps::Bool=false,
                    dimensions::Int=2, calc_mean::Bool=false, stokes::Bool=false,
                    sort_z::Bool=false, precision::Symbol=:fp64)
    (RM === nothing && !stokes) || error("Faraday rotation is not supported by the GPU path")
    dimensions in (2, 3) || return nothing
    if sort_z
        Pos, par_c = SPHtoGrid.center_particles(Pos, param)  # in place, as the reference
        sel = SPHtoGrid.filter_particles_in_image(Pos, par_c, true)
        q_sel = ndims(Bin_Quant) == 1 ? Bin_Quant[sel] : Bin_Quant[:, sel]
        return map_selected(Pos[:, sel], HSML[sel], M[sel], Rho[sel], q_sel, Weights[sel], par_c, kernel,
                            show_progress, reduce_image, return_both_maps, dimensions, calc_mean, precision)
    end
    T = (eltype(HSML) == Float32 && eltype(M) == Float32 && eltype(Rho) == Float32 &&
         eltype(Bin_Quant) == Float32 && eltype(Weights) == Float32) ? Float32 : Float64
    pos = eltype(Pos) <: Union{Float32,Float64} ? Pos : Float64.(Pos)
    hsml, m, rho, w = T.(HSML), T.(M), T.(Rho), T.(Weights)
    q = T.(Bin_Quant)
    N = length(M)
    nq = ndims(q) == 1 ? 1 : size(q, 1)
    P = param.Npixels[1]
    out = return_both_maps && dimensions == 2 ? zeros(Float64, P * P, nq + 1) :
          dimensions == 2 ? zeros(Float64, P, P, nq) : zeros(Float64, P, P, P)
    GC.@preserve pos hsml m rho w q out begin
        pt = SphgParticles(N, dtype_id(eltype(pos)), dtype_id(T), pointer(pos), 3, 1,
                           pointer(hsml), pointer(m), pointer(rho), pointer(w), pointer(q),
                           Int32(nq), Int32(0), ndims(q) == 1 ? 1 : nq, ndims(q) == 1 ? 0 : 1)
        kdim = hasfield(typeof(kernel), :dim) ? Int32(kernel.dim) : Int32(3)
        opt = SphgOptions(dimensions, kernel_id(kernel), kdim, reduce_image, return_both_maps,
                          calc_mean, precision === :fp32c ? 1 : 0, 0, 1, 1, 1, 0, 0, (0, 0, 0))
        st = SphgStats()
        status = ccall((:sphg_map, libsphgrid), Cint,
                       (Ptr{Cvoid}, Ref{SphgParams}, Ref{SphgOptions}, Ref{SphgParticles},
                        Ptr{Float64}, Ptr{Cvoid}, Ref{SphgStats}),
                       context(), SphgParams(param), opt, pt, pointer(out), C_NULL, st)
        status == 0 || error(unsafe_string(ccall((:sphg_last_error, libsphgrid), Cstring,
                                                 (Ptr{Cvoid},), context())))
    end
    pos === Pos || (Pos .= pos)  # the reference centres the caller's array in place
    show_progress && @info "Particles in image: $(st.n_mapped) / $N, deposits: $(st.deposits)"
    return out
end

# ------------------------------------------------------------------ map_it

struct SphgProjection
    kind::Int32          # 0 xy, 1 xz, 2 yz, 3 matrix
    reserved::Int32
    matrix::NTuple{9,Float64}  # row-major
end

"""
    map_it(pos_in, hsml, mass, rho, bin_q, weights=rho; param, kernel=WendlandC6(2),
           projection="xy", reduce_image=true, calc_mean=true, precision=:fp64)

The map of `map_it` (cic_interpolation.jl:314-380) on the GPU: the positions
are read through the projection ("xy", "xz", "yz" or three Euler angles in
degrees, RotXYZ as rotate_3D builds it) and `pos_in` is left intact.  Returns
the map; write it with the reference's `write_fits_image` as map_it does.
"""
function map_it(pos_in::Array{<:Real}, hsml, mass, rho, bin_q, weights=rho;
                param::mappingParameters, kernel::AbstractSPHKernel=WendlandC6(2),
                projection="xy", reduce_image::Bool=true, calc_mean::Bool=true,
                precision::Symbol=:fp64)
    T = (eltype(hsml) == Float32 && eltype(mass) == Float32 && eltype(rho) == Float32 &&
         eltype(bin_q) == Float32 && eltype(weights) == Float32) ? Float32 : Float64
    pos = eltype(pos_in) <: Union{Float32,Float64} ? pos_in : Float64.(pos_in)
    h, m, r, w, q = T.(hsml), T.(mass), T.(rho), T.(weights), T.(bin_q)
    N = length(m)
    nq = ndims(q) == 1 ? 1 : size(q, 1)
    P = param.Npixels[1]
    out = zeros(Float64, P, P, nq)
    zero9 = ntuple(_ -> 0.0, 9)
    proj = projection == "xy" ? SphgProjection(0, 0, zero9) :
           projection == "xz" ? SphgProjection(1, 0, zero9) :
           projection == "yz" ? SphgProjection(2, 0, zero9) :
           SphgProjection(3, 0, Tuple(vec(permutedims(Matrix(RotXYZ(deg2rad.(projection)...))))))
    GC.@preserve pos h m r w q out begin
        pt = SphgParticles(N, dtype_id(eltype(pos)), dtype_id(T), pointer(pos), 3, 1,
                           pointer(h), pointer(m), pointer(r), pointer(w), pointer(q),
                           Int32(nq), Int32(0), ndims(q) == 1 ? 1 : nq, ndims(q) == 1 ? 0 : 1)
        kdim = hasfield(typeof(kernel), :dim) ? Int32(kernel.dim) : Int32(3)
        # centre mode 2: read-only (map_it maps a copy of the positions)
        opt = SphgOptions(2, kernel_id(kernel), kdim, reduce_image, false, calc_mean,
                          precision === :fp32c ? 1 : 0, 0, 2, 1, 1, 0, 0, (0, 0, 0))
        st = SphgStats()
        status = ccall((:sphg_map_projected, libsphgrid), Cint,
                       (Ptr{Cvoid}, Ref{SphgParams}, Ref{SphgOptions}, Ref{SphgParticles},
                        Ref{SphgProjection}, Ptr{Float64}, Ptr{Cvoid}, Ref{SphgStats}),
                       context(), SphgParams(param), opt, pt, proj, pointer(out), C_NULL, st)
        status == 0 || error(unsafe_string(ccall((:sphg_last_error, libsphgrid), Cstring,
                                                 (Ptr{Cvoid},), context())))
    end
    return out
end

# -------------------------------------------------------------- healpix_map

struct SphgHealpixParams
    nside::Int64
    kernel::Int32
    kernel_dim::Int32
    calc_mean::Int32
    dtype::Int32
end

"""
    healpix_map(Pos, Hsml, M, Rho, Bin_q, Weights; center=[0.0, 0.0, 0.0],
                radius_limits=[0.0, Inf], Nside=1024, kernel, calc_mean=true)

The reference's `healpix_map` (healpix_interpolation/main.jl:92-227) with the
particle loop on the GPU in FP64: `filter_sort_particles` is the reference's
own (it centres `Pos` in place); the selected particles go to
`sphg_healpix_map`.  Returns `(allsky_map, weight_map)` as
`HealpixMap{Float64,RingOrder}`s.
"""
function healpix_map(Pos, Hsml, M, Rho, Bin_q, Weights; center::Vector{<:Real}=[0.0, 0.0, 0.0],
                     radius_limits::Vector{<:Real}=[0.0, Inf], Nside::Integer=1024,
                     kernel::AbstractSPHKernel, calc_mean::Bool=true, kwargs...)
    Healpix = Base.require(Base.PkgId(Base.UUID("9f4e344d-96bc-545a-84a3-ae6b9e1b672b"), "Healpix"))
    CUDA = Base.require(Base.PkgId(Base.UUID("052768ef-5323-5732-b1bb-66c8b64840ba"), "CUDA"))
    npix = 12 * Nside^2
    allsky = Healpix.HealpixMap{Float64,Healpix.RingOrder}(Nside)
    weight = Healpix.HealpixMap{Float64,Healpix.RingOrder}(Nside)
    (!calc_mean && iszero(sum(Bin_q))) && return allsky, weight
    pos, hsml, m, rho, q, w = SPHtoGrid.filter_sort_particles(Pos, Hsml, M, Rho, Bin_q, Weights,
                                                             center, radius_limits, calc_mean)
    d = map(a -> CUDA.CuArray{Float64}(a), (pos, hsml, m, rho, q, w))
    da, dw = CUDA.zeros(Float64, npix), CUDA.zeros(Float64, npix)
    ptr(a) = reinterpret(Ptr{Cvoid}, pointer(a))
    hp = SphgHealpixParams(Nside, kernel_id(kernel),
                           hasfield(typeof(kernel), :dim) ? Int32(kernel.dim) : Int32(3),
                           calc_mean, 1)
    st = SphgStats()
    s = ccall((:sphg_healpix_map, libsphgrid), Cint,
              (Ptr{Cvoid}, Ref{SphgHealpixParams}, Int64, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid},
               Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{SphgStats}),
              context(), hp, length(hsml), ptr(d[1]), ptr(d[2]), ptr(d[3]), ptr(d[4]), ptr(d[5]),
              ptr(d[6]), ptr(da), ptr(dw), C_NULL, st)
    s == 0 || error(unsafe_string(ccall((:sphg_last_error, libsphgrid), Cstring, (Ptr{Cvoid},), context())))
    allsky.pixels .= Array(da)
    weight.pixels .= Array(dw)
    return allsky, weight
end

# ---------------------------------------------------------------- adjoint

struct SphgGrads
    pos::Ptr{Cvoid}
    hsml::Ptr{Cvoid}
    mass::Ptr{Cvoid}
    rho::Ptr{Cvoid}
    weights::Ptr{Cvoid}
    bin_q::Ptr{Cvoid}
end

using ChainRulesCore: ChainRulesCore, NoTangent, unthunk

"""
    rrule(::typeof(sphMapping_differentiable), Pos, HSML, M, Rho, Bin_Quant, Weights; kw...)

ChainRulesCore rule of the GPU map (device arrays, `CuArray`s).  The forward
deposits into the raw accumulator (`raw_accumulator = 1`), reduces it with
`sphg_reduce`, and keeps the accumulator; the pullback calls `sphg_adjoint`,
which recomputes the kernel weights instead of storing the particle-pixel
list and returns dL/d(Pos, HSML, M, Rho, Bin_Quant, Weights).  `precision`
is the forward's, `adjoint_precision` (default: the same) the pullback's:
`:fp64`, or `:fp32c` (per-cell terms in FP32 with compensated sums, particles
whose sums cancel beyond the FP32 rounding estimate redone in FP64).
"""
function sphMapping_differentiable(Pos, HSML, M, Rho, Bin_Quant, Weights; param::mappingParameters,
                                   kernel::AbstractSPHKernel, dimensions::Int=2, reduce_image::Bool=true,
                                   precision::Symbol=:fp64, adjoint_precision::Symbol=precision)
    # outside automatic differentiation: the forward of the rule, pullback dropped
    out, _ = ChainRulesCore.rrule(sphMapping_differentiable, Pos, HSML, M, Rho, Bin_Quant, Weights;
                                  param=param, kernel=kernel, dimensions=dimensions,
                                  reduce_image=reduce_image, precision=precision,
                                  adjoint_precision=adjoint_precision)
    return out
end

function ChainRulesCore.rrule(::typeof(sphMapping_differentiable), Pos, HSML, M, Rho, Bin_Quant,
                              Weights; param::mappingParameters, kernel::AbstractSPHKernel,
                              dimensions::Int=2, reduce_image::Bool=true, precision::Symbol=:fp64,
                              adjoint_precision::Symbol=precision)
    CUDA = Base.require(Base.PkgId(Base.UUID("052768ef-5323-5732-b1bb-66c8b64840ba"), "CUDA"))
    T = eltype(HSML)
    N = length(M)
    nq = ndims(Bin_Quant) == 1 ? 1 : size(Bin_Quant, 1)
    P = param.Npixels[1]
    PD = dimensions == 2 ? P^2 : P^3
    raw = CUDA.zeros(Float64, PD * (nq + 1))
    out = dimensions == 2 ? CUDA.zeros(Float64, P, P, nq) : CUDA.zeros(Float64, P, P, P)
    kdim = hasfield(typeof(kernel), :dim) ? Int32(kernel.dim) : Int32(3)
    mkopt(raw_acc, prec=precision) = SphgOptions(dimensions, kernel_id(kernel), kdim, reduce_image, false, false,
                                                 prec === :fp32c ? 1 : 0, 0, 2, 1, 0, 0, raw_acc, (0, 0, 0))
    ptr(a) = reinterpret(Ptr{Cvoid}, pointer(a))
    pt = SphgParticles(N, dtype_id(eltype(Pos)), dtype_id(T), ptr(Pos), 3, 1, ptr(HSML), ptr(M),
                       ptr(Rho), ptr(Weights), ptr(Bin_Quant), Int32(nq), Int32(0),
                       ndims(Bin_Quant) == 1 ? 1 : nq, ndims(Bin_Quant) == 1 ? 0 : 1)
    st = SphgStats()
    s = ccall((:sphg_map, libsphgrid), Cint,
              (Ptr{Cvoid}, Ref{SphgParams}, Ref{SphgOptions}, Ref{SphgParticles}, Ptr{Cvoid},
               Ptr{Cvoid}, Ref{SphgStats}),
              context(), SphgParams(param), mkopt(1), pt, ptr(raw), C_NULL, st)
    s == 0 || error("sphg_map failed with status $s")
    s = ccall((:sphg_reduce, libsphgrid), Cint,
              (Ptr{Cvoid}, Ref{SphgParams}, Ref{SphgOptions}, Int32, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
              context(), SphgParams(param), mkopt(0), Int32(nq), ptr(raw), ptr(out), C_NULL)
    s == 0 || error("sphg_reduce failed with status $s")
    function pullback(dout)
        g = CUDA.CuArray{Float64}(unthunk(dout))
        dpos = CUDA.zeros(Float64, size(Pos))
        dh, dm, dr, dw = (CUDA.zeros(Float64, N) for _ in 1:4)
        dq = CUDA.zeros(Float64, size(Bin_Quant))
        gr = SphgGrads(ptr(dpos), ptr(dh), ptr(dm), ptr(dr), ptr(dw), ptr(dq))
        s = ccall((:sphg_adjoint, libsphgrid), Cint,
                  (Ptr{Cvoid}, Ref{SphgParams}, Ref{SphgOptions}, Ref{SphgParticles}, Ptr{Cvoid},
                   Ptr{Cvoid}, Ref{SphgGrads}, Ptr{Cvoid}),
                  context(), SphgParams(param), mkopt(0, adjoint_precision), pt, ptr(raw), ptr(g), gr, C_NULL)
        s == 0 || error("sphg_adjoint failed with status $s")
        return (NoTangent(), dpos, dh, dm, dr, dq, dw)
    end
    return out, pullback
end

end # module
