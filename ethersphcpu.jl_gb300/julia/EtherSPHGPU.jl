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
  given without `aabb` runs on the host at every check step, as the reference runs it
  (FluidWallSolve.jl:73-81): the steps run in chunks that end at check steps, the live
  fluid is downloaded, the closure deletes, and the survivors are uploaded again.

  With `staged_output = true` (the default when no host-side check is needed) the files
  are written by the library (sph_output_*): the state after an output step is copied on
  the device and written by a library thread while the next steps run; the files hold
  the same fields and groups as writeVTP's, in VTK's appended raw layout.

  Also here: `GPUScene` (a device-resident scene: step!, download!, probe via
  kernelValueInterpolation), `GPUBatch` (many scenes stepped together) and `serve`, the
  request loop that admits scenes by device footprint into running batches.
=#
module EtherSPHGPU

using EtherSPHCPU

export GPU, FP64, FP32Compensated, GPUScene, GPUBatch, SceneRequest, serve, step!, download!, probe, PlaneRules,
    stepAsync!, synchronize, stats, countPairs, timeStages, autotune!, setLaunchShape!, setStencilPruning!, sceneInfo,
    setBufferVelocity!

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

# solve variant of a wall group (SPH_SOLVE_*): FluidWallSolve, FluidThermostaticWallSolve,
# FluidVelocitySolve
solveCode(walls) = walls[1] isa ThermostaticWallParticle ? Int32(1) :
                   walls[1] isa StaticVelocityWallParticle ? Int32(3) : Int32(0)
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

function checkStatus(h, rc)
    if rc != 0
        msg = unsafe_string(ccall((:sph_last_error, libsph), Cstring, (Ptr{Cvoid},), h))
        error("EtherSPHGPU error $rc: $msg")
    end
    return nothing
end

# dim x n (an empty group gives a 0 x 0 matrix: the library reads no element of it)
stack(ps, f) = isempty(ps) ? zeros(0, 0) : reduce(hcat, [collect(Float64, getfield(p, f)) for p in ps])

function uploadFluid(h, fluid)
    x, v = stack(fluid, :x_vec_), stack(fluid, :v_vec_)
    sc(f) = Float64[getfield(p, f) for p in fluid]
    th = eltype(fluid) <: ThermalLiquidParticle
    t, kappa, cp = th ? (sc(:t_), sc(:kappa_), sc(:cp_)) : (C_NULL, C_NULL, C_NULL)
    checkStatus(h, ccall((:sph_upload_fluid, libsph), Int32,
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
    checkStatus(h, ccall((:sph_upload_walls, libsph), Int32,
        (Ptr{Cvoid}, Int32, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h, kind, length(walls), x, n, gap, t, kappa, v))
end

# Copy the live particles back into the Julia vector (deleteat! for removed ones).
function downloadFluid!(h, fluid)
    isempty(fluid) && return nothing  # nothing left to update (every particle was deleted)
    cap = length(fluid)
    dim = length(fluid[1].x_vec_)
    x, v = zeros(dim, cap), zeros(dim, cap)
    rho, p, c, m, gap = zeros(cap), zeros(cap), zeros(cap), zeros(cap), zeros(cap)
    th = eltype(fluid) <: ThermalLiquidParticle
    t = th ? zeros(cap) : C_NULL
    n = Ref{Int64}(0)
    checkStatus(h, ccall((:sph_download_fluid, libsph), Int32,
        (Ptr{Cvoid}, Int64, Ref{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h, cap, n, x, v, rho, p, c, m, gap, t, C_NULL, C_NULL))
    ids = zeros(Int64, cap)
    checkStatus(h, ccall((:sph_download_ids, libsph), Int32, (Ptr{Cvoid}, Int64, Ref{Int64}, Ptr{Int64}), h, cap, n, ids))
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

function openOutput(h, vtp_io::VTPIO)
    syms = [lstrip(String(x), ':') for x in vtp_io.field_symbols_]
    names = String[x for x in vtp_io.field_names_]
    checkStatus(h, ccall((:sph_output_open, libsph), Int32,
        (Ptr{Cvoid}, Cstring, Cstring, Cstring, Int32, Int32, Ptr{Cstring}, Ptr{Cstring}, Cstring),
        h, vtp_io.dir_path_, vtp_io.file_name_, vtp_io.file_suffix_, Int32(vtp_io.step_digit_), Int32(length(syms)),
        syms, names, C_NULL))
end

outputWrite(h, file_step, t) =
    checkStatus(h, ccall((:sph_output_write, libsph), Int32, (Ptr{Cvoid}, Int64, Float64), h, file_step, t))
outputFlush(h) = checkStatus(h, ccall((:sph_output_flush, libsph), Int32, (Ptr{Cvoid},), h))

function runSolve!(solve_code, fluid, wall_groups, kernel, model, td, vtp_io, check, aabb, precision, domain,
    periodic_x, staged_output, autotune = false)
    if domain === nothing
        pts = reduce(hcat, [stack(g, :x_vec_) for g in [[fluid]; wall_groups] if !isempty(g)])
        pad = 2 * kernel.influence_radius_
        domain = (vec(minimum(pts; dims = 2)) .- pad, vec(maximum(pts; dims = 2)) .+ pad)
    end
    prm = Ref(makeParams(kernel, model, td, solve_code, precision, aabb, domain, periodic_x))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    nw = sum(length, wall_groups; init = 0)
    checkStatus(C_NULL, ccall((:sph_create, libsph), Int32, (Ref{SphParams}, Int64, Int64, Ref{Ptr{Cvoid}}),
        prm, length(fluid), nw, h))
    host_check = aabb === nothing && check !== defaultCheck  # a closure: run on the host at check steps
    staged = staged_output && !host_check
    try
        foreach(g -> uploadWalls(h[], g), wall_groups)
        uploadFluid(h[], fluid)
        if autotune && precision == FP32Compensated  # launch shape picked on this scene
            checkStatus(h[], ccall((:sph_autotune, libsph), Int32, (Ptr{Cvoid}, Int32, Ptr{Int32}), h[], Int32(3),
                C_NULL))
        end
        if staged
            openOutput(h[], vtp_io)
            outputWrite(h[], 0, 0.0)
        else
            assureDirPathExist(vtp_io)
            writeVTP(0, 0.0, vtp_io, [[fluid]; wall_groups])
        end
        nextStop(step, interval) = (div(step - 1, interval) + 1) * interval
        step = 1
        while step <= td.total_step_
            # chunks end at output steps, and at check steps when the closure runs here
            last = min(td.total_step_, nextStop(step, td.output_interval_))
            host_check && (last = min(last, nextStop(step, td.check_interval_)))
            fresh = false  # `fluid` holds the device state
            try
                checkStatus(h[], ccall((:sph_step, libsph), Int32, (Ptr{Cvoid}, Int64, Int64), h[], step, last - step + 1))
            catch e  # FluidWallSolve.jl:130-133: report, write the state of the failing step, continue
                println(e)
                println("Error at step: ", last)
                if staged
                    outputWrite(h[], last, last * td.dt_)
                else
                    downloadFluid!(h[], fluid)
                    fresh = true
                    writeVTP(last, last * td.dt_, vtp_io, [[fluid]; wall_groups])
                end
            end
            if host_check && isCheckStep(last, td)  # deleteat!(fluid, !check) (FluidWallSolve.jl:73-81)
                fresh || downloadFluid!(h[], fluid)
                n_before = length(fluid)
                deleteat!(fluid, findall(p -> !check(p), fluid))
                length(fluid) != n_before && uploadFluid(h[], fluid)
                fresh = true
            end
            if isOutputStep(last, td)
                if staged  # the library copies the state and writes while the next steps run
                    outputWrite(h[], div(last, td.output_interval_), last * td.dt_)
                else
                    fresh || downloadFluid!(h[], fluid)
                    writeVTP(div(last, td.output_interval_), last * td.dt_, vtp_io, [[fluid]; wall_groups])
                end
            end
            step = last + 1
        end
        staged && outputFlush(h[])
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
    periodic_x::Bool = false, staged_output::Bool = true, autotune::Bool = false)::Nothing
    code = solveCode(wall_particles)
    return runSolve!(code, fluid_particles, [wall_particles], smooth_kernel, wc_lm, dr_fti_forward_euler, vtp_io,
        check, aabb, precision, domain, periodic_x, staged_output, autotune)
end

# FluidCompulsiveThermostaticWallSolve.jl:154-233
function EtherSPHCPU.solve!(::GPU, fluid_particles::AbstractVector{<:FluidParticle},
    wall_particles::AbstractVector{<:WallParticle},
    thermostatic_wall_particles::AbstractVector{<:ThermostaticWallParticle}, smooth_kernel::SmoothKernel,
    th_wc_lm::ThermalWeaklyCompressibleLiquidModel,
    dr_fti_forward_euler::DensityReinitializedFixedTimeIntervalForwardEuler, vtp_io::VTPIO;
    check::Function = defaultCheck, aabb = nothing, precision = FP64, domain = nothing,
    staged_output::Bool = true, autotune::Bool = false)::Nothing
    return runSolve!(Int32(2), fluid_particles, [wall_particles, thermostatic_wall_particles], smooth_kernel,
        th_wc_lm, dr_fti_forward_euler, vtp_io, check, aabb, precision, domain, false, staged_output, autotune)
end

# ---------------------------------------------------------------- inlet / outlet
# Mirror of SphBufferRules (include/ethersph_gpu.h).
struct SphBufferRules
    inlet_normal::NTuple{3, Float64}
    inlet_offset::Float64
    inlet_shift::NTuple{3, Float64}
    outlet_normal::NTuple{3, Float64}
    outlet_offset::Float64
    drop_normal::NTuple{3, Float64}
    drop_offset::Float64
end

"""
    PlaneRules(; inlet = (normal, offset), shift, outlet = (normal, offset), drop = (normal, offset))

The keyword closures of the inlet/outlet solve! as planes: a particle passes a check when
normal . x > offset (inletIntoCalculationDomainCheck(p) = p.x_vec_[1] > x0 is
inlet = ([1, 0], x0)); an inlet particle that entered the fluid moves by `shift`
(inletIntoCalculationDomainModify).
"""
PlaneRules(; inlet, shift, outlet, drop) = SphBufferRules(pad3(inlet[1]), Float64(inlet[2]), pad3(shift),
    pad3(outlet[1]), Float64(outlet[2]), pad3(drop[1]), Float64(drop[2]))

function uploadBuffers(h, rules::SphBufferRules, inlet, outlet, capacity)
    f(g, k) = isempty(g) ? Float64[] : (k === :x_vec_ || k === :v_vec_ ? stack(g, k) : Float64[getfield(p, k) for p in g])
    checkStatus(h, ccall((:sph_upload_buffers, libsph), Int32,
        (Ptr{Cvoid}, Ref{SphBufferRules}, Int64, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64,
         Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h, Ref(rules), capacity, length(inlet), f(inlet, :x_vec_), f(inlet, :v_vec_), f(inlet, :rho_), f(inlet, :p_),
        f(inlet, :c_), f(inlet, :mass_), f(inlet, :gap_), length(outlet), f(outlet, :x_vec_), f(outlet, :v_vec_),
        f(outlet, :rho_), f(outlet, :p_), f(outlet, :c_), f(outlet, :mass_), f(outlet, :gap_)))
end

# The inlet (which = 0) or outlet (1) particles back into `group` (resized to the device's).
function downloadBuffers!(h, which, group, dim)
    n = Ref{Int64}(0)
    ccall((:sph_download_buffers, libsph), Int32, (Ptr{Cvoid}, Int32, Int64, Ref{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h, Int32(which), 0, n, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL)  # the count
    x, v = zeros(dim, n[]), zeros(dim, n[])
    rho, p, c, m, gap = zeros(n[]), zeros(n[]), zeros(n[]), zeros(n[]), zeros(n[])
    checkStatus(h, ccall((:sph_download_buffers, libsph), Int32,
        (Ptr{Cvoid}, Int32, Int64, Ref{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h, Int32(which), n[], n, x, v, rho, p, c, m, gap))
    proto = group[1]
    while length(group) < n[]
        push!(group, deepcopy(proto))
    end
    resize!(group, n[])
    for (i, pt) in enumerate(group)
        pt.x_vec_ .= view(x, :, i)
        pt.v_vec_ .= view(v, :, i)
        pt.rho_, pt.p_, pt.c_, pt.mass_, pt.gap_ = rho[i], p[i], c[i], m[i], gap[i]
    end
    return group
end

"""
    setBufferVelocity!(h, which, v::Matrix{Float64})

Overwrite the inlet (0) or outlet (1) velocities (dim x n, in their order): what the
example's user_defined_function does between steps (PoiseuilleFlow2D.jl:152-167).
"""
setBufferVelocity!(h, which, v::AbstractMatrix) = checkStatus(h, ccall((:sph_set_buffer_velocity, libsph), Int32,
    (Ptr{Cvoid}, Int32, Int64, Ptr{Float64}), h, Int32(which), size(v, 2), Matrix{Float64}(v)))

# FluidInletOutletWallSolve.jl:264-340.  user_defined_function(h, t) runs on the host
# every `udf_interval` steps (the reference: after every step), with the handle for
# setBufferVelocity!.
function EtherSPHCPU.solve!(::GPU, fluid_particles::AbstractVector{<:FluidParticle},
    inlet_fluid_particles::AbstractVector{<:FluidParticle}, outlet_fluid_particles::AbstractVector{<:FluidParticle},
    wall_particles::AbstractVector{<:WallParticle}, smooth_kernel::SmoothKernel,
    wc_lm::WeaklyCompressibleLiquidModel, dr_fti_forward_euler::DensityReinitializedFixedTimeIntervalForwardEuler,
    vtp_io::VTPIO; rules::SphBufferRules, user_defined_function = nothing, udf_interval::Int = 1,
    precision = FP64, domain = nothing, fluid_capacity::Int = 2 * length(fluid_particles) +
    64 * length(inlet_fluid_particles), buffer_capacity::Int = length(inlet_fluid_particles) +
    length(outlet_fluid_particles) + fluid_capacity)::Nothing
    td = dr_fti_forward_euler
    groups = [fluid_particles, inlet_fluid_particles, outlet_fluid_particles, wall_particles]
    if domain === nothing
        pts = reduce(hcat, [stack(g, :x_vec_) for g in groups if !isempty(g)])
        pad = 2 * smooth_kernel.influence_radius_
        domain = (vec(minimum(pts; dims = 2)) .- pad, vec(maximum(pts; dims = 2)) .+ pad)
    end
    prm = Ref(makeParams(smooth_kernel, wc_lm, td, Int32(4), precision, nothing, domain, false))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    checkStatus(C_NULL, ccall((:sph_create, libsph), Int32, (Ref{SphParams}, Int64, Int64, Ref{Ptr{Cvoid}}),
        prm, fluid_capacity, length(wall_particles), h))
    dim = length(fluid_particles[1].x_vec_)
    pull!() = begin
        downloadFluidAll!(h[], fluid_particles)
        downloadBuffers!(h[], 0, inlet_fluid_particles, dim)
        downloadBuffers!(h[], 1, outlet_fluid_particles, dim)
    end
    try
        uploadWalls(h[], wall_particles)
        uploadFluid(h[], fluid_particles)
        uploadBuffers(h[], rules, inlet_fluid_particles, outlet_fluid_particles, buffer_capacity)
        assureDirPathExist(vtp_io)
        writeVTP(0, 0.0, vtp_io, groups)
        step = 1
        while step <= td.total_step_
            stop = step
            while stop < td.total_step_ && stop % udf_interval != 0 && !isOutputStep(stop, td)
                stop += 1
            end
            checkStatus(h[], ccall((:sph_step, libsph), Int32, (Ptr{Cvoid}, Int64, Int64), h[], step, stop - step + 1))
            user_defined_function === nothing || user_defined_function(h[], stop * td.dt_)
            if isOutputStep(stop, td)
                pull!()
                writeVTP(div(stop, td.output_interval_), stop * td.dt_, vtp_io, groups)
            end
            step = stop + 1
        end
        pull!()
    finally
        ccall((:sph_destroy, libsph), Int32, (Ptr{Cvoid},), h[])
    end
    return nothing
end

# The live fluid into the vector, growing it for particles that came from the inlet
# (every field from the device, in ascending id).
function downloadFluidAll!(h, fluid)
    n = Ref{Int64}(0)
    ccall((:sph_download_fluid, libsph), Int32, (Ptr{Cvoid}, Int64, Ref{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h, 0, n, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL)  # the count
    dim = length(fluid[1].x_vec_)
    x, v = zeros(dim, n[]), zeros(dim, n[])
    rho, p, c, m, gap = zeros(n[]), zeros(n[]), zeros(n[]), zeros(n[]), zeros(n[])
    checkStatus(h, ccall((:sph_download_fluid, libsph), Int32,
        (Ptr{Cvoid}, Int64, Ref{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h, n[], n, x, v, rho, p, c, m, gap, C_NULL, C_NULL, C_NULL))
    proto = fluid[1]
    while length(fluid) < n[]
        push!(fluid, deepcopy(proto))
    end
    resize!(fluid, n[])
    for (i, pt) in enumerate(fluid)
        pt.x_vec_ .= view(x, :, i)
        pt.v_vec_ .= view(v, :, i)
        pt.rho_, pt.p_, pt.c_, pt.mass_, pt.gap_ = rho[i], p[i], c[i], m[i], gap[i]
    end
    return fluid
end

# ---------------------------------------------------------------- a device-resident scene
"""
    GPUScene(fluid, wall_groups, kernel, model, td; precision, domain, aabb, periodic_x)

One scene held on the device (sph_create + uploads).  `step!(s, first, n)` runs steps
first .. first+n-1 of eachStep!; `download!(s, fluid)` copies the live particles back
(deleteat! for removed ones); `kernelValueInterpolation(points, s, field)` interpolates a
fluid field at points on the device (VTPToDataFrame.jl:93-142); `close(s)` frees it.
"""
mutable struct GPUScene
    h::Ptr{Cvoid}
    dim::Int
end

function GPUScene(fluid, wall_groups, kernel, model, td; precision = FP64, domain = nothing, aabb = nothing,
    periodic_x::Bool = false)
    if domain === nothing
        pts = reduce(hcat, [stack(g, :x_vec_) for g in [[fluid]; wall_groups] if !isempty(g)])
        pad = 2 * kernel.influence_radius_
        domain = (vec(minimum(pts; dims = 2)) .- pad, vec(maximum(pts; dims = 2)) .+ pad)
    end
    code = isThermal(model) ? (length(wall_groups) > 1 ? Int32(2) : Int32(1)) : solveCode(wall_groups[1])
    prm = Ref(makeParams(kernel, model, td, code, precision, aabb, domain, periodic_x))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    checkStatus(C_NULL, ccall((:sph_create, libsph), Int32, (Ref{SphParams}, Int64, Int64, Ref{Ptr{Cvoid}}),
        prm, length(fluid), sum(length, wall_groups; init = 0), h))
    s = GPUScene(h[], Int(kernel.dim_))
    foreach(g -> uploadWalls(s.h, g), wall_groups)
    uploadFluid(s.h, fluid)
    finalizer(close, s)
    return s
end

function Base.close(s::GPUScene)
    if s.h != C_NULL
        ccall((:sph_destroy, libsph), Int32, (Ptr{Cvoid},), s.h)
        s.h = C_NULL
    end
    return nothing
end

step!(s::GPUScene, first_step::Integer, nsteps::Integer) =
    checkStatus(s.h, ccall((:sph_step, libsph), Int32, (Ptr{Cvoid}, Int64, Int64), s.h, first_step, nsteps))
download!(s::GPUScene, fluid) = downloadFluid!(s.h, fluid)

"""
    stepAsync!(s, first_step, nsteps); synchronize(s)

sph_step_async / sph_synchronize: enqueue steps on the scene's stream and return at once;
`synchronize` waits and reports a non-finite state or an overflow as an error.
"""
stepAsync!(s::GPUScene, first_step::Integer, nsteps::Integer) =
    checkStatus(s.h, ccall((:sph_step_async, libsph), Int32, (Ptr{Cvoid}, Int64, Int64), s.h, first_step, nsteps))
synchronize(s::GPUScene) = checkStatus(s.h, ccall((:sph_synchronize, libsph), Int32, (Ptr{Cvoid},), s.h))

# Mirror of SphStats (include/ethersph_gpu.h).
struct SphStats
    n_fluid::Int64
    n_wall::Int64
    steps_done::Int64
    total_mass::Float64
    kinetic_energy::Float64
    max_speed::Float64
    status_flags::Int32
    reserved0::Int32
end

"""
    stats(s) -> SphStats

FP64 reductions on the device: live particles, total mass, kinetic energy, max speed.
"""
function stats(s::GPUScene)
    out = Ref{SphStats}()
    checkStatus(s.h, ccall((:sph_stats, libsph), Int32, (Ptr{Cvoid}, Ref{SphStats}), s.h, out))
    return out[]
end

"""
    countPairs(s) -> (fluid_pairs, wall_pairs)

Unique fluid pairs (i < j, the CellListMap half-list convention) and fluid-wall pairs
within r_cut at the current positions.
"""
function countPairs(s::GPUScene)
    a, b = Ref{Int64}(0), Ref{Int64}(0)
    checkStatus(s.h, ccall((:sph_count_pairs, libsph), Int32, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}), s.h, a, b))
    return (a[], b[])
end

"""
    timeStages(s; reps = 10) -> Vector{Float64}

Milliseconds per stage (cell hash + count, scan, placement, continuity, momentum,
Shepard), CUDA events on the scene's stream; the state is left unchanged.
"""
function timeStages(s::GPUScene; reps::Integer = 10)
    ms = zeros(Float64, 6)
    checkStatus(s.h, ccall((:sph_time_stages, libsph), Int32, (Ptr{Cvoid}, Int32, Ptr{Float64}), s.h, Int32(reps), ms))
    return ms
end

"""
    autotune!(s; reps = 3) -> NTuple{4, Int32}

sph_autotune: the FP32-compensated form's launch shape picked on the scene's live state.
"""
function autotune!(s::GPUScene; reps::Integer = 3)
    out = zeros(Int32, 4)
    checkStatus(s.h, ccall((:sph_autotune, libsph), Int32, (Ptr{Cvoid}, Int32, Ptr{Int32}), s.h, Int32(reps), out))
    return Tuple(out)
end

setLaunchShape!(s::GPUScene, shape::Vector{Int32}) =
    checkStatus(s.h, ccall((:sph_set_launch_shape, libsph), Int32, (Ptr{Cvoid}, Ptr{Int32}), s.h, shape))
setStencilPruning!(s::GPUScene, on::Bool) =
    checkStatus(s.h, ccall((:sph_set_stencil_pruning, libsph), Int32, (Ptr{Cvoid}, Int32), s.h, Int32(on)))

"""The cudaStream_t (as a pointer) the scene launches on, for CUDA-event timing."""
function stream(s::GPUScene)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    checkStatus(s.h, ccall((:sph_get_stream, libsph), Int32, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}), s.h, out))
    return out[]
end

"""The library's ABI version (SPH_ABI_VERSION)."""
abiVersion() = ccall((:sph_version, libsph), Int32, ())

const probeCodes = Dict(:rho_ => 0, :p_ => 1, :c_ => 2, :t_ => 6, :mass_ => 7, "Density" => 0, "Pressure" => 1,
    "SoundSpeed" => 2, "VelocityX" => 3, "VelocityY" => 4, "VelocityZ" => 5, "Temperature" => 6, "Mass" => 7)

"""
    probe(s::GPUScene, points::Matrix{Float64}, fields; none_value = NaN) -> Matrix

SPH interpolation of fluid fields (symbols such as :rho_ or column names such as
"VelocityX") at the columns of `points` (dim x n); one row per field.
"""
function probe(s::GPUScene, points::AbstractMatrix, fields; none_value::Float64 = NaN)
    pts = Matrix{Float64}(points)
    codes = Int32[probeCodes[f] for f in fields]
    out = zeros(Float64, size(pts, 2), length(codes))  # column-major: out[:, k] is field k
    checkStatus(s.h, ccall((:sph_probe, libsph), Int32,
        (Ptr{Cvoid}, Int64, Ptr{Float64}, Int32, Ptr{Int32}, Float64, Ptr{Float64}),
        s.h, size(pts, 2), pts, Int32(length(codes)), codes, none_value, out))
    return permutedims(out)
end

# kernelValueInterpolation(points, view, field, kernel, indices) of VTPToDataFrame.jl,
# evaluated on the live device state of `s` (fluid particles) instead of a VTP file.
EtherSPHCPU.kernelValueInterpolation(points::Matrix, s::GPUScene, field; none_value::Float64 = NaN) =
    vec(probe(s, points, [field]; none_value = none_value))

# ---------------------------------------------------------------- batches and serving
"""
    GPUBatch(prototype::SphParams, particles, cells, walls, scenes)

A batch handle (sph_batch_create): scenes of one dim / kernel / solve / form share the
kernel launches; capacities are the device budget.
"""
mutable struct GPUBatch
    h::Ptr{Cvoid}
end

function GPUBatch(prototype::SphParams, particles::Integer, cells::Integer, walls::Integer, scenes::Integer)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    checkStatus(C_NULL, ccall((:sph_batch_create, libsph), Int32,
        (Ref{SphParams}, Int64, Int64, Int64, Int32, Ref{Ptr{Cvoid}}),
        Ref(prototype), particles, cells, walls, Int32(scenes), h))
    b = GPUBatch(h[])
    finalizer(close, b)
    if prototype.precision == FP32Compensated  # the serving loop's shape: the neighbour list, two lanes
        setLaunchShape!(b, Int32[-1, LANES_LIST + 2, -1, 128])
    end
    return b
end

"""
    setLaunchShape!(b, shape)

sph_set_launch_shape: (continuity lanes, momentum lanes, Shepard lanes, block size) of the
FP32-compensated form; momentum lanes LANES_LIST + t read the neighbour list.
"""
setLaunchShape!(b::GPUBatch, shape::Vector{Int32}) =
    checkStatus(b.h, ccall((:sph_set_launch_shape, libsph), Int32, (Ptr{Cvoid}, Ptr{Int32}), b.h, shape))

const LANES_LIST = Int32(16)  # SPH_LANES_LIST

function Base.close(b::GPUBatch)
    if b.h != C_NULL
        ccall((:sph_destroy, libsph), Int32, (Ptr{Cvoid},), b.h)
        b.h = C_NULL
    end
    return nothing
end

function freeSlots(b::GPUBatch)
    out = zeros(Int64, 4)
    checkStatus(b.h, ccall((:sph_batch_free, libsph), Int32, (Ptr{Cvoid}, Ptr{Int64}), b.h, out))
    return (particles = out[1], cells = out[2], walls = out[3], scenes = out[4])
end

function footprint(prm::SphParams, n_fluid::Integer, n_wall::Integer)
    out = zeros(Int64, 3)
    checkStatus(C_NULL, ccall((:sph_scene_footprint, libsph), Int32, (Ref{SphParams}, Int64, Int64, Ptr{Int64}),
        Ref(prm), n_fluid, n_wall, out))
    return (particles = out[1], cells = out[2], walls = out[3])
end

function addScene!(b::GPUBatch, prm::SphParams, first_step::Integer, nsteps::Integer, fluid, wall_groups)
    x, v = stack(fluid, :x_vec_), stack(fluid, :v_vec_)
    sc(f) = Float64[getfield(p, f) for p in fluid]
    th = fluid[1] isa ThermalLiquidParticle
    t, kappa, cp = th ? (sc(:t_), sc(:kappa_), sc(:cp_)) : (C_NULL, C_NULL, C_NULL)
    walls = reduce(vcat, wall_groups; init = WallParticle[])
    nw = length(walls)
    kinds = Int32[wallCode(w) for w in walls]
    wx = nw > 0 ? stack(walls, :x_vec_) : zeros(0, 0)
    wn = nw > 0 ? stack(walls, :normal_vec_) : zeros(0, 0)
    wgap = Float64[w.gap_ for w in walls]
    wt = Float64[w isa ThermostaticWallParticle ? w.t_ : 0.0 for w in walls]
    wk = Float64[w isa ThermostaticWallParticle ? w.kappa_ : 0.0 for w in walls]
    dim = length(fluid[1].x_vec_)
    wv = nw > 0 ? reduce(hcat, [w isa StaticVelocityWallParticle ? collect(Float64, w.v_vec_) : zeros(dim)
                               for w in walls]) : zeros(0, 0)
    id = Ref{Int32}(-1)
    checkStatus(b.h, ccall((:sph_batch_add_scene, libsph), Int32,
        (Ptr{Cvoid}, Ref{SphParams}, Int64, Int64, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{Int32},
         Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{Int32}),
        b.h, Ref(prm), first_step, nsteps, length(fluid), x, v, sc(:rho_), sc(:p_), sc(:c_), sc(:mass_), sc(:gap_),
        t, kappa, cp, nw, kinds, wx, wn, wgap, wt, wk, wv, id))
    return Int(id[])
end

stepBatch!(b::GPUBatch, nsteps::Integer) =
    checkStatus(b.h, ccall((:sph_batch_step, libsph), Int32, (Ptr{Cvoid}, Int64), b.h, nsteps))
synchronize(b::GPUBatch) = checkStatus(b.h, ccall((:sph_synchronize, libsph), Int32, (Ptr{Cvoid},), b.h))

"""
    sceneInfo(b, id) -> (n_fluid, steps_done, finished, next_step)

sph_batch_scene_info: the scene's live particles, steps run, whether its step budget is
done, and the number of its next step.
"""
function sceneInfo(b::GPUBatch, id::Integer)
    info = zeros(Int64, 4)
    checkStatus(b.h, ccall((:sph_batch_scene_info, libsph), Int32, (Ptr{Cvoid}, Int32, Ptr{Int64}), b.h, Int32(id), info))
    return (n_fluid = info[1], steps_done = info[2], finished = info[3] != 0, next_step = info[4])
end
retire!(b::GPUBatch, id::Integer) =
    checkStatus(b.h, ccall((:sph_batch_retire, libsph), Int32, (Ptr{Cvoid}, Int32), b.h, Int32(id)))

function downloadScene!(b::GPUBatch, id::Integer, fluid)
    cap = length(fluid)
    dim = length(fluid[1].x_vec_)
    x, v = zeros(dim, cap), zeros(dim, cap)
    rho, p, c, m, gap = zeros(cap), zeros(cap), zeros(cap), zeros(cap), zeros(cap)
    th = fluid[1] isa ThermalLiquidParticle
    t, kappa, cp = th ? (zeros(cap), zeros(cap), zeros(cap)) : (C_NULL, C_NULL, C_NULL)
    n = Ref{Int64}(0)
    checkStatus(b.h, ccall((:sph_batch_download_scene, libsph), Int32,
        (Ptr{Cvoid}, Int32, Int64, Ref{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        b.h, Int32(id), cap, n, x, v, rho, p, c, m, gap, t, kappa, cp))
    # the survivors in their original order; every field comes from the device, so the
    # first n structs are reused whichever particles were deleted
    resize!(fluid, n[])
    for (i, pt) in enumerate(fluid)
        pt.x_vec_ .= view(x, :, i)
        pt.v_vec_ .= view(v, :, i)
        pt.rho_ = rho[i]
        pt.p_ = p[i]
        pt.c_ = c[i]
        pt.mass_ = m[i]
        pt.gap_ = gap[i]
        if th
            pt.t_ = t[i]
            pt.kappa_ = kappa[i]
            pt.cp_ = cp[i]
        end
    end
    return fluid
end

"""
    SceneRequest(t_arrival, fluid, wall_groups, kernel, model, td; precision, domain, aabb, periodic_x)

A scene to serve: it arrives at `t_arrival` seconds and runs td.total_step_ steps.
"""
struct SceneRequest
    t_arrival::Float64
    fluid::Any
    wall_groups::Any
    params::SphParams
    nsteps::Int
end

function SceneRequest(t_arrival, fluid, wall_groups, kernel, model, td; precision = FP32Compensated,
    domain = nothing, aabb = nothing, periodic_x::Bool = false)
    if domain === nothing
        pts = reduce(hcat, [stack(g, :x_vec_) for g in [[fluid]; wall_groups] if !isempty(g)])
        pad = 2 * kernel.influence_radius_
        domain = (vec(minimum(pts; dims = 2)) .- pad, vec(maximum(pts; dims = 2)) .+ pad)
    end
    code = isThermal(model) ? (length(wall_groups) > 1 ? Int32(2) : Int32(1)) : solveCode(wall_groups[1])
    prm = makeParams(kernel, model, td, code, precision, aabb, domain, periodic_x)
    return SceneRequest(Float64(t_arrival), fluid, wall_groups, prm, Int(td.total_step_))
end

"""
    serve(requests, batches::Dict{Int, GPUBatch}; bundle = 10) -> (results, wall_s, particle_steps)

The request loop: requests (sorted by arrival) join the queue of their dimension when
they arrive; a queued scene is admitted into its batch as soon as its footprint fits the
batch's free particle slots, cell run, wall run and scene slot; every bundle advances all
resident scenes together; finished scenes are downloaded into their fluid vectors and
retired, which frees room for the queue.  `results` holds (request, t_admit, t_done) with
times in seconds from the start; latency = t_done - t_arrival.
"""
function serve(requests::Vector{SceneRequest}, batches::Dict{Int, GPUBatch}; bundle::Int = 10)
    pending = sort(requests; by = r -> r.t_arrival)
    queues = Dict(d => SceneRequest[] for d in keys(batches))
    active = Dict{Tuple{Int, Int}, Any}()
    results = Tuple{SceneRequest, Float64, Float64}[]
    particle_steps = 0
    t0 = time()
    while !isempty(pending) || !isempty(active) || any(!isempty, values(queues))
        now = time() - t0
        while !isempty(pending) && pending[1].t_arrival <= now
            r = popfirst!(pending)
            push!(queues[Int(r.params.dim)], r)
        end
        for (dim, q) in queues
            b = batches[dim]
            while !isempty(q)
                r = q[1]
                need = footprint(r.params, length(r.fluid), sum(length, r.wall_groups; init = 0))
                fr = freeSlots(b)
                (need.particles <= fr.particles && need.cells <= fr.cells && need.walls <= fr.walls &&
                 fr.scenes >= 1) || break
                popfirst!(q)
                id = addScene!(b, r.params, 1, r.nsteps, r.fluid, r.wall_groups)
                active[(dim, id)] = [r, time() - t0, r.nsteps, length(r.fluid)]
            end
        end
        if isempty(active)
            isempty(pending) || sleep(max(0.0, min(0.01, pending[1].t_arrival - (time() - t0))))
            continue
        end
        running = unique(first.(collect(keys(active))))
        foreach(d -> stepBatch!(batches[d], bundle), running)
        foreach(d -> synchronize(batches[d]), running)
        t_now = time() - t0
        for key in collect(keys(active))
            rec = active[key]
            n = min(bundle, rec[3])
            particle_steps += n * rec[4]
            rec[3] -= n
            if rec[3] <= 0
                dim, id = key
                downloadScene!(batches[dim], id, rec[1].fluid)
                retire!(batches[dim], id)
                push!(results, (rec[1], rec[2], t_now))
                delete!(active, key)
            end
        end
    end
    return results, time() - t0, particle_steps
end

end # module
