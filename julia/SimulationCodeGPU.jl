# SimulationCodeGPU.jl -- binds SimulationCode.jl's molecular-dynamics hot
# path to libsimmd (include/simmd.h) by ccall.  ArrayStruct, ParameterStruct,
# OutputStruct and the potential / system types of SimulationCode.jl are used
# unchanged; the functions below take their place on the hot path:
#
#   initialize_neighbor_struct (src/DataStructs.jl:349)  -> GPUNeighborList
#   update_neighbor_lists!     (src/NeighborLists.jl:24) -> gpu_update_neighbor_lists!
#   calculate_new_forces!      (src/MD.jl:262)           -> gpu_calculate_new_forces!
#   do_time_step               (src/MD.jl:429, 499)      -> gpu_do_time_steps!
#   calculate_full_energy      (src/AuxiliaryFunctions.jl:22) -> gpu_calculate_full_energy
#   find_inherent_structure    (src/InherentStructure.jl:5)   -> gpu_find_inherent_structure!
#   save_data's copy           (src/Dump.jl:60-88)       -> gpu_dump_async / gpu_dump_wait
#
# Julia is not installed where libsimmd was built, so this module has not
# been executed; the same entry points are exercised from Python ctypes by
# the repository's tests.  Point SIMMD_LIB at simulationcode_gb300/_lib/libsimmd.so.
module SimulationCodeGPU

export GPUNeighborList, gpu_update_neighbor_lists!, gpu_calculate_new_forces!, gpu_do_time_steps!,
       gpu_calculate_full_energy, gpu_find_inherent_structure!, gpu_dump_async, gpu_dump_wait,
       gpu_perform_molecular_dynamics!, gpu_check_conversions

const libsimmd = get(ENV, "SIMMD_LIB", "libsimmd.so")

const SIMMD_FP64 = Int32(0)
const SIMMD_FP32_SPLIT = Int32(1)
const SIMMD_ERR_NOT_CONVERGED = Cint(10)

# simmd_params, field for field
struct SimmdParams
    dims::Int32; potential::Int32; dynamics::Int32; precision::Int32
    N::Int64
    box_size::Float64; force_cutoff2::Float64; skin::Float64; verlet_force_cutoff::Float64
    lj_eps::Float64; lj_sigma::Float64; lj_Uc::Float64
    b_c0::Float64; b_c2::Float64; b_c4::Float64; b_zeta::Float64
    kBT::Float64; gamma::Float64; dt::Float64; m::Float64
    rescale_temperature::Int32; max_neighbors::Int32
    seed::UInt64
end

# simmd_stats
struct SimmdStats
    steps_done::Int64; rebuilds::Int64; noise_draws::Int64
    max_neighbors::Int32; max_count::Int32; overflow::Int32; nonfinite::Int32
    epot::Float64; virial::Float64; ekin::Float64
    list_entries::Int64
end

function check(st::Cint)
    st == 0 && return nothing
    msg = unsafe_string(ccall((:simmd_last_error, libsimmd), Cstring, ()))
    error("libsimmd status $st: $msg")
end

pot_code(U) = nameof(typeof(U)) === :LJ ? Int32(0) : Int32(1)
dyn_code(S) = nameof(typeof(S)) === :Newtonian ? Int32(0) : (nameof(typeof(S)) === :Langevin ? Int32(1) : Int32(2))

function SimmdParams(p, skin, force_cutoff; precision=SIMMD_FP64, maxneighbours=200)
    U, S = p.interaction_potential, p.system
    lj = pot_code(U) == 0
    brownian = dyn_code(S) == 2
    newtonian = dyn_code(S) == 0
    SimmdParams(Int32(S.dims), pot_code(U), dyn_code(S), precision, p.N, p.box_size, p.force_cutoff2, skin,
                force_cutoff,
                lj ? U.ϵ : 1.0, lj ? U.σ : 1.0, lj ? U.Uc : 0.0,
                lj ? 0.0 : U.c0, lj ? 0.0 : U.c2, lj ? 0.0 : U.c4, lj ? 0.0 : U.ζ,
                S.kBT, newtonian ? 0.0 : S.γ, S.Δt, brownian ? 1.0 : S.m,
                (newtonian && S.rescale_temperature) ? Int32(1) : Int32(0), Int32(maxneighbours),
                UInt64(p.random_seed))
end

flat(x) = reinterpret(reshape, Float64, x)   # Vector{SVector{d,Float64}} -> d x N

mutable struct GPUNeighborList
    ctx::Ptr{Cvoid}
    rebuilds_seen::Int64
end

"""initialize_neighbor_struct: a device context holding the state and lists"""
function GPUNeighborList(arrays, parameters, skin, force_cutoff; precision=SIMMD_FP64, maxneighbours=200)
    prm = Ref(SimmdParams(parameters, skin, force_cutoff; precision, maxneighbours))
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:simmd_create, libsimmd), Cint, (Ref{SimmdParams}, Ref{Ptr{Cvoid}}), prm, ctx))
    GC.@preserve arrays check(ccall((:simmd_upload, libsimmd), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        ctx[], pointer(flat(arrays.r_array)), pointer(flat(arrays.v_array)), pointer(flat(arrays.F_array)),
        pointer(arrays.D_array), C_NULL))
    nl = GPUNeighborList(ctx[], 0)
    finalizer(x -> ccall((:simmd_destroy, libsimmd), Cint, (Ptr{Cvoid},), x.ctx), nl)
    nl
end

function to_device!(nl::GPUNeighborList, arrays)
    GC.@preserve arrays check(ccall((:simmd_set_state, libsimmd), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        nl.ctx, pointer(flat(arrays.r_array)), pointer(flat(arrays.v_array)), pointer(flat(arrays.F_array)),
        C_NULL))
end

function from_device!(nl::GPUNeighborList, arrays)
    GC.@preserve arrays check(ccall((:simmd_download, libsimmd), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        nl.ctx, pointer(flat(arrays.r_array)), pointer(flat(arrays.v_array)), pointer(flat(arrays.F_array)),
        C_NULL))
end

function stats(nl::GPUNeighborList)
    st = Ref{SimmdStats}()
    check(ccall((:simmd_stats_get, libsimmd), Cint, (Ptr{Cvoid}, Ref{SimmdStats}), nl.ctx, st))
    st[]
end

function count_rebuilds!(nl::GPUNeighborList, output)
    rb = stats(nl).rebuilds
    output.N_neighbor_list_rebuilds += rb - nl.rebuilds_seen
    nl.rebuilds_seen = rb
end

"""update_neighbor_lists! (src/NeighborLists.jl:24)"""
function gpu_update_neighbor_lists!(arrays, output, nl::GPUNeighborList)
    to_device!(nl, arrays)
    check(ccall((:simmd_rebuild, libsimmd), Cint, (Ptr{Cvoid},), nl.ctx))
    count_rebuilds!(nl, output)
end

"""calculate_new_forces! (src/MD.jl:262); noise: the d x N deviates of this
call (arrays.random_displacement after randn!) or nothing for Philox"""
function gpu_calculate_new_forces!(arrays, nl::GPUNeighborList; noise=nothing)
    to_device!(nl, arrays)
    GC.@preserve arrays noise check(ccall((:simmd_forces, libsimmd), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), nl.ctx,
        noise === nothing ? C_NULL : pointer(flat(noise)), pointer(flat(arrays.F_array))))
end

"""do_time_step x nsteps (src/MD.jl:429, 499) in one call; the state stays on
the device and is copied back at the end"""
function gpu_do_time_steps!(arrays, output, nl::GPUNeighborList, nsteps::Integer)
    to_device!(nl, arrays)
    check(ccall((:simmd_step, libsimmd), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}), nl.ctx, nsteps, C_NULL))
    from_device!(nl, arrays)
    count_rebuilds!(nl, output)
end

"""calculate_full_energy (src/AuxiliaryFunctions.jl:22)"""
function gpu_calculate_full_energy(arrays, nl::GPUNeighborList)
    to_device!(nl, arrays)
    e = Ref(0.0)
    check(ccall((:simmd_energy, libsimmd), Cint, (Ptr{Cvoid}, Ref{Float64}, Ptr{Float64}, Ptr{Float64}),
                nl.ctx, e, C_NULL, C_NULL))
    e[]
end

"""find_inherent_structure (src/InherentStructure.jl:5); returns iterations"""
function gpu_find_inherent_structure!(arrays, nl::GPUNeighborList; tolerance=1e-6, max_iterations=10^6,
                                      max_step_size=0.001, dt=0.005)
    to_device!(nl, arrays)
    it = Ref{Int64}(0)
    st = ccall((:simmd_inherent_structure, libsimmd), Cint,
               (Ptr{Cvoid}, Float64, Int64, Float64, Float64, Ref{Int64}),
               nl.ctx, tolerance, max_iterations, max_step_size, dt, it)
    from_device!(nl, arrays)
    st == SIMMD_ERR_NOT_CONVERGED && error("Not converged")
    check(st)
    it[]
end

"""queue the copy of r, v, F into page-locked host buffers (d x N Float64
matrices registered with simmd_host_register) while later steps run"""
function gpu_dump_async(nl::GPUNeighborList, r::Matrix{Float64}, v::Matrix{Float64}, F::Matrix{Float64})
    check(ccall((:simmd_dump_async, libsimmd), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                nl.ctx, 0, pointer(r), pointer(v), pointer(F)))
end

gpu_dump_wait(nl::GPUNeighborList) = check(ccall((:simmd_dump_wait, libsimmd), Cint, (Ptr{Cvoid},), nl.ctx))

"""the step loop of perform_molecular_dynamics! (src/MD.jl:704-715): with the
no-op callback the steps between dump / log steps run in one device call;
`on_host_step(arrays, step)` is called at those steps with the state copied
back (the reference's save_data / print_log_data go there)"""
function gpu_perform_molecular_dynamics!(arrays, parameters, output, nl::GPUNeighborList, host_steps;
                                         on_host_step=(a, s) -> nothing)
    stops = sort(unique(filter(s -> output.steps_done < s <= parameters.N_steps,
                               vcat(collect(host_steps), parameters.N_steps))))
    for s in stops
        gpu_do_time_steps!(arrays, output, nl, s - output.steps_done)
        output.steps_done = s
        on_host_step(arrays, s)
    end
end

"""device self-check: mismatches of the split kernels' bit-level float <->
double conversions and grid index against the hardware (0 expected)"""
function gpu_check_conversions(n::Integer=1 << 24, seed::Integer=1)
    bad = Ref{Int64}(-1)
    check(ccall((:simmd_check_conversions, libsimmd), Cint, (Int64, UInt64, Ref{Int64}), n, seed, bad))
    bad[]
end

end # module
