#=
  EtherSPHGPU.jl — GPU solve! methods for EtherSPHCPU.jl models.

  Adds methods to EtherSPHCPU.solve! that take a leading `GPU()` marker and otherwise
  the same arguments as the CPU methods (src/Solve/FluidWallSolve.jl:85-93,
  FluidThermostaticWallSolve.jl:127-135, FluidCompulsiveThermostaticWallSolve.jl:154-165,
  FluidVelocitySolve.jl:104-112).  The particle vectors are marshalled into plain
  arrays, the time loop runs in libethersph_gpu.so (include/ethersph_gpu.h), and at every
  output step the state is copied back into the particle structs and written with the
  unchanged writeVTP, so the VTP files have the reference's format.

  The `check::Function` keyword cannot run on the device; pass `aabb = (lo, hi)` (a
  particle is deleted at a check step when a coordinate is > hi or < lo), which is what
  the examples' check functions express (CollapseDry.jl:119-127).  A `check` function
  given without `aabb` is applied on the host at output steps only.
=#
module EtherSPHGPU

using EtherSPHCPU

export GPU, FP64, FP32Compensated

const libsph = joinpath(@__DIR__, "..", "lib", "libethersph_gpu.so")

struct GPU end
const FP64 = Int32(0)
const FP32Compensated = Int32(1)

# Mirror of SphParams (include/ethersph_gpu.h); field order and types must match.
struct SphParams
    dim::Int32
    kernel::Int32
    solve::Int32
    precision::Int32
    influence_radius::Float64
    h::Float64
    sigma::Float64
    kernel_0::Float64
    rho_0::Float64
    c_0::Float64
    p_0::Float64
    gamma::Int32
    thermal::Int32
    b::Float64
    mu_0::Float64
    nu_0::Float64
    body_force::NTuple{3, Float64}
    t_0::Float64
    kappa_0::Float64
    cp::Float64
    beta::Float64
    dt::Float64
    total_step::Int64
    output_interval::Int64
    check_interval::Int64
    density_reinitialized_interval::Int64
    check_enabled::Int32
    periodic_x::Int32
    check_lo::NTuple{3, Float64}
    check_hi::NTuple{3, Float64}
    domain_lo::NTuple{3, Float64}
    domain_hi::NTuple{3, Float64}
    nan_check::Int32
    cell_subdivision::Int32
end

kernelCode(::CubicSpline) = Int32(0)
kernelCode(::Gaussian) = Int32(1)
kernelCode(::WendlandC2) = Int32(2)
kernelCode(::WendlandC4) = Int32(3)

wallCode(::CompulsiveWallParticle) = Int32(0)
wallCode(::StaticVelocityWallParticle) = Int32(1)
wallCode(::ThermostaticWallParticle) = Int32(2)

pad3(v) = ntuple(k -> k <= length(v) ? Float64(v[k]) : 0.0, 3)
isThermal(m) = m isa ThermalWeaklyCompressibleLiquidModel

function makeParams(kernel, model, td, solve_code, precision, aabb, domain, periodic_x)
    lo, hi = aabb === nothing ? ((-Inf, -Inf, -Inf), (Inf, Inf, Inf)) : (pad3(aabb[1]), pad3(aabb[2]))
    if aabb !== nothing
        lo = ntuple(k -> k <= length(aabb[1]) ? Float64(aabb[1][k]) : -Inf, 3)
        hi = ntuple(k -> k <= length(aabb[2]) ? Float64(aabb[2][k]) : Inf, 3)
    end
    th = isThermal(model)
    return SphParams(
        Int32(kernel.dim_), kernelCode(kernel), solve_code, precision,
        kernel.influence_radius_, kernel.h_, kernel.sigma_, kernel.kernel_0_,
        model.rho_0_, model.c_0_, model.p_0_, Int32(model.gamma_), Int32(th),
        model.b_, model.mu_0_, model.nu_0_, pad3(model.body_force_vec_),
        th ? model.t_0_ : 0.0, th ? model.kappa_0_ : 0.0, th ? model.cp_ : 0.0, th ? model.beta_ : 0.0,
        td.dt_, Int64(td.total_step_), Int64(td.output_interval_), Int64(td.check_interval_),
        Int64(td.density_reinitialized_interval_),
        Int32(aabb !== nothing), Int32(periodic_x), lo, hi, pad3(domain[1]), pad3(domain[2]), Int32(1), Int32(0),
    )
end

function check(h, rc)
    if rc != 0
        msg = unsafe_string(ccall((:sph_last_error, libsph), Cstring, (Ptr{Cvoid},), h))
        error("EtherSPHGPU error $rc: $msg")
    end
    return nothing
end

stack(ps, f) = reduce(hcat, [collect(Float64, getfield(p, f)) for p in ps])  # dim x n

function uploadFluid(h, fluid)
    x, v = stack(fluid, :x_vec_), stack(fluid, :v_vec_)
    sc(f) = Float64[getfield(p, f) for p in fluid]
    th = fluid[1] isa ThermalLiquidParticle
    t, kappa, cp = th ? (sc(:t_), sc(:kappa_), sc(:cp_)) : (C_NULL, C_NULL, C_NULL)
    check(h, ccall((:sph_upload_fluid, libsph), Int32,
        (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h, length(fluid), x, v, sc(:rho_), sc(:p_), sc(:c_), sc(:mass_), sc(:gap_), t, kappa, cp))
end

function uploadWalls(h, walls)
    isempty(walls) && return nothing
    x, n = stack(walls, :x_vec_), stack(walls, :normal_vec_)
    gap = Float64[w.gap_ for w in walls]
    kind = wallCode(walls[1])
    t = kind == 2 ? Float64[w.t_ for w in walls] : C_NULL
    kappa = kind == 2 ? Float64[w.kappa_ for w in walls] : C_NULL
    v = kind == 1 ? stack(walls, :v_vec_) : C_NULL
    check(h, ccall((:sph_upload_walls, libsph), Int32,
        (Ptr{Cvoid}, Int32, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h, kind, length(walls), x, n, gap, t, kappa, v))
end

# Copy the live particles back into the Julia vector (deleteat! for removed ones).
function downloadFluid!(h, fluid)
    cap = length(fluid)
    dim = length(fluid[1].x_vec_)
    x, v = zeros(dim, cap), zeros(dim, cap)
    rho, p, c, m, gap = zeros(cap), zeros(cap), zeros(cap), zeros(cap), zeros(cap)
    th = fluid[1] isa ThermalLiquidParticle
    t = th ? zeros(cap) : C_NULL
    n = Ref{Int64}(0)
    check(h, ccall((:sph_download_fluid, libsph), Int32,
        (Ptr{Cvoid}, Int64, Ref{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h, cap, n, x, v, rho, p, c, m, gap, t, C_NULL, C_NULL))
    ids = zeros(Int64, cap)
    check(h, ccall((:sph_download_ids, libsph), Int32, (Ptr{Cvoid}, Int64, Ref{Int64}, Ptr{Int64}), h, cap, n, ids))
    keep = falses(cap)
    keep[ids[1:n[]] .+ 1] .= true
    deleteat!(fluid, findall(.!keep))
    for (i, pt) in enumerate(fluid)
        pt.x_vec_ .= view(x, :, i)
        pt.v_vec_ .= view(v, :, i)
        pt.rho_ = rho[i]
        pt.p_ = p[i]
        pt.c_ = c[i]
        th && (pt.t_ = t[i])
    end
    return nothing
end

function runSolve!(solve_code, fluid, wall_groups, kernel, model, td, vtp_io, check, aabb, precision, domain,
    periodic_x)
    if domain === nothing
        pts = reduce(hcat, [stack(g, :x_vec_) for g in [[fluid]; wall_groups] if !isempty(g)])
        pad = 2 * kernel.influence_radius_
        domain = (vec(minimum(pts; dims = 2)) .- pad, vec(maximum(pts; dims = 2)) .+ pad)
    end
    prm = Ref(makeParams(kernel, model, td, solve_code, precision, aabb, domain, periodic_x))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    nw = sum(length, wall_groups; init = 0)
    check(C_NULL, ccall((:sph_create, libsph), Int32, (Ref{SphParams}, Int64, Int64, Ref{Ptr{Cvoid}}),
        prm, length(fluid), nw, h))
    try
        foreach(g -> uploadWalls(h[], g), wall_groups)
        uploadFluid(h[], fluid)
        assureDirPathExist(vtp_io)
        writeVTP(0, 0.0, vtp_io, [[fluid]; wall_groups])
        step = 1
        while step <= td.total_step_
            last = min(td.total_step_, (div(step - 1, td.output_interval_) + 1) * td.output_interval_)
            try
                check(h[], ccall((:sph_step, libsph), Int32, (Ptr{Cvoid}, Int64, Int64), h[], step, last - step + 1))
            catch e  # FluidWallSolve.jl:130-134: report and continue
                println(e)
                println("Error at step: ", last)
            end
            if isOutputStep(last, td)
                downloadFluid!(h[], fluid)
                if aabb === nothing && check !== defaultCheck
                    deleteat!(fluid, findall(p -> !check(p), fluid))
                    uploadFluid(h[], fluid)
                end
                writeVTP(div(last, td.output_interval_), last * td.dt_, vtp_io, [[fluid]; wall_groups])
            end
            step = last + 1
        end
        downloadFluid!(h[], fluid)
    finally
        ccall((:sph_destroy, libsph), Int32, (Ptr{Cvoid},), h[])
    end
    return nothing
end

# FluidWallSolve.jl:85-140 (or FluidVelocitySolve.jl for StaticVelocityWallParticle walls,
# FluidThermostaticWallSolve.jl for ThermostaticWallParticle walls)
function EtherSPHCPU.solve!(::GPU, fluid_particles::AbstractVector{<:FluidParticle},
    wall_particles::AbstractVector{<:WallParticle}, smooth_kernel::SmoothKernel,
    wc_lm::WeaklyCompressibleLiquidModel, dr_fti_forward_euler::DensityReinitializedFixedTimeIntervalForwardEuler,
    vtp_io::VTPIO; check::Function = defaultCheck, aabb = nothing, precision = FP64, domain = nothing,
    periodic_x::Bool = false)::Nothing
    code = wall_particles[1] isa ThermostaticWallParticle ? Int32(1) :
           wall_particles[1] isa StaticVelocityWallParticle ? Int32(3) : Int32(0)
    return runSolve!(code, fluid_particles, [wall_particles], smooth_kernel, wc_lm, dr_fti_forward_euler, vtp_io,
        check, aabb, precision, domain, periodic_x)
end

# FluidCompulsiveThermostaticWallSolve.jl:154-233
function EtherSPHCPU.solve!(::GPU, fluid_particles::AbstractVector{<:FluidParticle},
    wall_particles::AbstractVector{<:WallParticle},
    thermostatic_wall_particles::AbstractVector{<:ThermostaticWallParticle}, smooth_kernel::SmoothKernel,
    th_wc_lm::ThermalWeaklyCompressibleLiquidModel,
    dr_fti_forward_euler::DensityReinitializedFixedTimeIntervalForwardEuler, vtp_io::VTPIO;
    check::Function = defaultCheck, aabb = nothing, precision = FP64, domain = nothing)::Nothing
    return runSolve!(Int32(2), fluid_particles, [wall_particles, thermostatic_wall_particles], smooth_kernel,
        th_wc_lm, dr_fti_forward_euler, vtp_io, check, aabb, precision, domain, false)
end

end # module
