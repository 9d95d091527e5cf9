# SimulationCodeGPU.jl -- runs SimulationCode.jl's molecular-dynamics hot path
# in libsimmd (include/simmd.h) by ccall, as methods of SimulationCode's own
# generic functions.  ArrayStruct, ParameterStruct, OutputStruct, the
# potential and system types and perform_molecular_dynamics! itself are used
# unchanged; only the neighbour-list object changes type:
#
#   neighborlist = SimulationCode.initialize_neighbor_struct(skin, box_size, rc, N,
#                                                            arrays.D_array, dims, SimulationCodeGPU.GPU())
#   SimulationCode.perform_molecular_dynamics!(arrays, parameters, output, neighborlist)
#
# Methods added for a GPUNeighborList (reference definitions in brackets):
#   initialize_neighbor_struct  (src/DataStructs.jl:349)      -> a device context (created on first use)
#   update_neighbor_lists!      (src/NeighborLists.jl:24)     -> simmd_rebuild
#   calculate_new_forces!       (src/MD.jl:262)               -> simmd_forces
#   do_time_step                (src/MD.jl:429, 499)          -> simmd_step, steps batched (below)
#   run_short_MD_equilibration! (src/MD.jl:579)               -> one simmd_step call
#   calculate_full_energy       (src/AuxiliaryFunctions.jl:22) -> simmd_energy
#   compute_potential_energy!   (src/AuxiliaryFunctions.jl:186) -> simmd_potential_energy_array
#   print_log_data              (src/MD.jl:610)               -> E_pot_test from lists built afresh on the device
#   find_inherent_structure     (src/InherentStructure.jl:5)  -> simmd_inherent_structure
#   do_MC_step!                 (src/MC.jl:139)               -> simmd_mc_sweeps, sweeps batched as steps
#
# Step batching: when the callback is `nocallback` (or the list was made
# with batch_steps=true, the caller's promise that its callback reads no
# state), do_time_step records the step and the recorded steps run in one
# device call (CUDA-graph step loop) at the next step whose state the host
# sees: a dump step (save_data), a log step (print_log_data), the last step,
# or any method above.  With any other callback each step runs and is copied
# back before the callback, as the reference does.
#
# Julia is not installed where libsimmd was built, so this module has not
# been executed; the same protocol is implemented and tested against the
# oracle in simulationcode_gb300/md.py (tests/test_gpu_driver.py).  Point
# SIMMD_LIB at simulationcode_gb300/_lib/libsimmd.so.
module SimulationCodeGPU

using SimulationCode
import SimulationCode: initialize_neighbor_struct, update_neighbor_lists!, calculate_new_forces!, do_time_step,
                       run_short_MD_equilibration!, calculate_full_energy, compute_potential_energy!,
                       print_log_data, find_inherent_structure, do_MC_step!, logdata
using SimulationCode: Newtonian, Langevin, Brownian

export GPU, GPUNeighborList, nocallback, gpu_dump_async, gpu_dump_wait, gpu_check_conversions,
       gpu_energy_virial_noalloc!, gpu_set_prune!

const libsimmd = get(ENV, "SIMMD_LIB", "libsimmd.so")

const SIMMD_FP64 = Int32(0)
const SIMMD_FP32_SPLIT = Int32(1)
const SIMMD_ERR_NOT_CONVERGED = Cint(10)
const SIMMD_NOALLOC_MAX_N = 1048576

"""device marker: the trailing argument of initialize_neighbor_struct that
puts the neighbour list (and the hot path) on the GPU"""
struct GPU
    precision::Int32
    maxneighbours::Int
    batch_steps::Bool
end
GPU(; precision=SIMMD_FP64, maxneighbours=200, batch_steps=false) = GPU(precision, maxneighbours, batch_steps)

"""the no-op callback; with it, steps between dump and log steps are batched"""
nocallback(x...) = nothing

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
    st == SIMMD_ERR_NOT_CONVERGED && error("Not converged")
    error("libsimmd status $st: $msg")
end

pot_code(U) = nameof(typeof(U)) === :LJ ? Int32(0) : Int32(1)
dyn_code(S) = S isa Newtonian ? Int32(0) : (S isa Langevin ? Int32(1) : Int32(2))

function SimmdParams(p, skin, force_cutoff; precision=SIMMD_FP64, maxneighbours=200)
    U, S = p.interaction_potential, p.system
    lj = pot_code(U) == 0
    brownian = S isa Brownian
    newtonian = S isa Newtonian
    SimmdParams(Int32(S.dims), pot_code(U), dyn_code(S), precision, p.N, p.box_size, p.force_cutoff2, skin,
                force_cutoff,
                lj ? U.ϵ : 1.0, lj ? U.σ : 1.0, lj ? U.Uc : 0.0,
                lj ? 0.0 : U.c0, lj ? 0.0 : U.c2, lj ? 0.0 : U.c4, lj ? 0.0 : U.ζ,
                S.kBT, newtonian ? 0.0 : S.γ, S.Δt, brownian ? 1.0 : S.m,
                (newtonian && S.rescale_temperature) ? Int32(1) : Int32(0), Int32(maxneighbours),
                UInt64(p.random_seed))
end

flat(x) = reinterpret(reshape, Float64, x)   # Vector{SVector{d,Float64}} -> d x N

"""NeighborListStruct on the device: the lists, displacements and cell data
live in a libsimmd context; the reference's fields are read through exports"""
mutable struct GPUNeighborList
    skin_distance::Float64
    force_cutoff::Float64
    N::Int
    dims::Int
    dev::GPU
    ctx::Ptr{Cvoid}
    prm::SimmdParams
    rebuilds_seen::Int64
    pending::Int64          # recorded steps not yet run on the device
    output::Any             # the OutputStruct of the recorded steps
    pending_mc::Int64       # recorded MC sweeps
    mc_args::Tuple{Float64,Float64}   # their (max_MC_displacement, swap_probability)
    mc_seen::Vector{Int64}  # move counters already added to the OutputStruct
    mc_dE_seen::Float64
end

"""initialize_neighbor_struct(skin, L, rc, N, D, dims, GPU()): the device
neighbour list; the context is created at the first call that carries the
ArrayStruct and ParameterStruct"""
function initialize_neighbor_struct(skin_distance, box_size, force_cutoff, N, D_array, dims, dev::GPU;
                                    maxneighbours=dev.maxneighbours)
    (dims == 2 || dims == 3) || error("To be implemented")
    nl = GPUNeighborList(skin_distance, force_cutoff, N, dims, GPU(dev.precision, maxneighbours, dev.batch_steps),
                         C_NULL, SimmdParams(ntuple(_ -> 0, 23)...), 0, 0, nothing, 0, (0.0, 0.0), zeros(Int64, 4), 0.0)
    finalizer(x -> x.ctx == C_NULL || ccall((:simmd_destroy, libsimmd), Cint, (Ptr{Cvoid},), x.ctx), nl)
    nl
end

function ensure!(nl::GPUNeighborList, arrays, parameters)
    nl.ctx != C_NULL && return nl
    nl.prm = SimmdParams(parameters, nl.skin_distance, nl.force_cutoff; precision=nl.dev.precision,
                         maxneighbours=nl.dev.maxneighbours)
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:simmd_create, libsimmd), Cint, (Ref{SimmdParams}, Ref{Ptr{Cvoid}}), Ref(nl.prm), ctx))
    nl.ctx = ctx[]
    GC.@preserve arrays check(ccall((:simmd_upload, libsimmd), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        nl.ctx, pointer(flat(arrays.r_array)), pointer(flat(arrays.v_array)), pointer(flat(arrays.F_array)),
        pointer(arrays.D_array), C_NULL))
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
    out = output === nothing ? nl.output : output
    out === nothing || (out.N_neighbor_list_rebuilds += rb - nl.rebuilds_seen)
    nl.rebuilds_seen = rb
end

# run the recorded steps plus `extra` from the host state of the last
# copy-back, then copy back
function run_steps!(nl::GPUNeighborList, arrays, output, extra)
    n = nl.pending + extra
    nl.pending = 0
    n == 0 && return nothing
    to_device!(nl, arrays)
    check(ccall((:simmd_step, libsimmd), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}), nl.ctx, n, C_NULL))
    from_device!(nl, arrays)
    count_rebuilds!(nl, output)
end

# run the recorded MC sweeps plus `extra`, then copy back r, D and the move
# counters (output.potential_energy += the accepted moves' dE)
function run_sweeps!(nl::GPUNeighborList, arrays, output, extra)
    n = nl.pending_mc + extra
    nl.pending_mc = 0
    n == 0 && return nothing
    to_device!(nl, arrays)
    check(ccall((:simmd_mc_sweeps, libsimmd), Cint, (Ptr{Cvoid}, Int64, Float64, Float64),
                nl.ctx, n, nl.mc_args[1], nl.mc_args[2]))
    from_device!(nl, arrays)
    GC.@preserve arrays check(ccall((:simmd_download_diameters, libsimmd), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}),
                                    nl.ctx, 0, pointer(arrays.D_array)))
    counts = zeros(Int64, 4)
    dE = Ref(0.0)
    check(ccall((:simmd_mc_stats, libsimmd), Cint, (Ptr{Cvoid}, Int32, Ptr{Int64}, Ref{Float64}),
                nl.ctx, 0, counts, dE))
    out = output === nothing ? nl.output : output
    if out !== nothing
        d = counts .- nl.mc_seen
        out.N_translations_accepted += d[1]; out.N_translations_total += d[2]
        out.N_swaps_accepted += d[3]; out.N_swaps_total += d[4]
        out.potential_energy += dE[] - nl.mc_dE_seen
    end
    nl.mc_seen = counts
    nl.mc_dE_seen = dE[]
    count_rebuilds!(nl, output)
end

# before any other device operation: recorded steps first, then the host state
function begin!(nl::GPUNeighborList, arrays, parameters, output)
    ensure!(nl, arrays, parameters)
    nl.pending > 0 && run_steps!(nl, arrays, output, 0)
    nl.pending_mc > 0 && run_sweeps!(nl, arrays, output, 0)
    to_device!(nl, arrays)
end

"""do_MC_step! (src/MC.jl:139-156) on the device: translation and swap
moves, the chain serial as in the reference; sweeps batched with the no-op
callback until the host sees the state (dump, log or last step)"""
function do_MC_step!(arrays, parameters, output, nl::GPUNeighborList, swap_probability)
    ensure!(nl, arrays, parameters)
    nl.pending > 0 && run_steps!(nl, arrays, output, 0)
    args = (Float64(parameters.max_MC_displacement), Float64(swap_probability))
    if nl.pending_mc > 0 && args != nl.mc_args
        run_sweeps!(nl, arrays, output, 0)
    end
    nl.mc_args = args
    if batching(nl, parameters)
        nl.output = output
        after = output.steps_done + 1    # steps_done advances after this call
        di = parameters.dump_info
        if !((di.save && after in di.when_to_save_array) || logdata(after) || after > parameters.N_steps)
            nl.pending_mc += 1
            return nothing
        end
    end
    run_sweeps!(nl, arrays, output, 1)
end

batching(nl::GPUNeighborList, parameters) = nl.dev.batch_steps || parameters.callback === nocallback

function host_sees(parameters, step)
    di = parameters.dump_info
    (di.save && step in di.when_to_save_array) || logdata(step) || step >= parameters.N_steps
end

function update_neighbor_lists!(arrays, parameters, output, nl::GPUNeighborList)
    begin!(nl, arrays, parameters, output)
    check(ccall((:simmd_rebuild, libsimmd), Cint, (Ptr{Cvoid},), nl.ctx))
    from_device!(nl, arrays)
    count_rebuilds!(nl, output)
end

function calculate_new_forces!(arrays, parameters, nl::GPUNeighborList)
    begin!(nl, arrays, parameters, nothing)
    GC.@preserve arrays check(ccall((:simmd_forces, libsimmd), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
                                    nl.ctx, C_NULL, pointer(flat(arrays.F_array))))
end

function gpu_step!(arrays, parameters, output, nl::GPUNeighborList)
    ensure!(nl, arrays, parameters)
    if batching(nl, parameters)
        nl.output = output
        if !host_sees(parameters, output.steps_done + 1)   # steps_done advances after this call
            nl.pending += 1
            return nothing
        end
        return run_steps!(nl, arrays, output, 1)
    end
    begin!(nl, arrays, parameters, output)
    check(ccall((:simmd_step, libsimmd), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}), nl.ctx, 1, C_NULL))
    from_device!(nl, arrays)
    count_rebuilds!(nl, output)
end

do_time_step(arrays, parameters, output, nl::GPUNeighborList, ::Union{Newtonian,Langevin}) =
    gpu_step!(arrays, parameters, output, nl)
do_time_step(arrays, parameters, output, nl::GPUNeighborList, ::Brownian) = gpu_step!(arrays, parameters, output, nl)

function run_short_MD_equilibration!(arrays, parameters, output, nl::GPUNeighborList)
    update_neighbor_lists!(arrays, parameters, output, nl)
    println("Performing short time MD equilibration")
    n = parameters.N_MD_equilibration_steps
    n > 0 || return nothing
    begin!(nl, arrays, parameters, output)
    check(ccall((:simmd_step, libsimmd), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}), nl.ctx, n, C_NULL))
    from_device!(nl, arrays)
    count_rebuilds!(nl, output)
end

function calculate_full_energy(arrays, parameters, nl::GPUNeighborList)
    begin!(nl, arrays, parameters, nothing)
    e = Ref(0.0)
    check(ccall((:simmd_energy, libsimmd), Cint, (Ptr{Cvoid}, Ref{Float64}, Ptr{Float64}, Ptr{Float64}),
                nl.ctx, e, C_NULL, C_NULL))
    e[]
end

function compute_potential_energy!(arrays, parameters, output, nl::GPUNeighborList)
    begin!(nl, arrays, parameters, output)
    GC.@preserve arrays check(ccall((:simmd_potential_energy_array, libsimmd), Cint, (Ptr{Cvoid}, Ptr{Float64}),
                                    nl.ctx, pointer(arrays.potential_energy_array)))
end

"""E_pot_test: the energy of the current positions from lists built afresh
in a temporary context, independent of the running lists"""
function energy_fresh_lists(arrays, nl::GPUNeighborList)
    tmp = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:simmd_create, libsimmd), Cint, (Ref{SimmdParams}, Ref{Ptr{Cvoid}}), Ref(nl.prm), tmp))
    try
        GC.@preserve arrays check(ccall((:simmd_upload, libsimmd), Cint,
            (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
            tmp[], pointer(flat(arrays.r_array)), C_NULL, C_NULL, pointer(arrays.D_array), C_NULL))
        e = Ref(0.0)
        check(ccall((:simmd_energy, libsimmd), Cint, (Ptr{Cvoid}, Ref{Float64}, Ptr{Float64}, Ptr{Float64}),
                    tmp[], e, C_NULL, C_NULL))
        return e[]
    finally
        ccall((:simmd_destroy, libsimmd), Cint, (Ptr{Cvoid},), tmp[])
    end
end

"""print_log_data (src/MD.jl:610-650) with E_pot_test from the device;
q4/q6 need the host lists and are left out (q_cutoff must be 0)"""
function print_log_data(arrays, parameters, output, nl::GPUNeighborList, start_time)
    parameters.q_cutoff > 0.0 && error("q4/q6 are not on the GPU path: set q_cutoff = 0")
    remaining_time = SimulationCode.estimated_remaining_time(output.steps_done, start_time, parameters.N_steps)
    output.potential_energy = calculate_full_energy(arrays, parameters, nl)
    if typeof(parameters.system) !== Brownian
        SimulationCode.find_kinetic_energy(arrays, parameters, output)
    else
        output.kinetic_energy = 0.0
    end
    SimulationCode.calculate_F2_self!(arrays, parameters, output)
    energy_no_neigh = energy_fresh_lists(arrays, nl)
    println("$(output.steps_done)/$(parameters.N_steps), ETA = $(round(remaining_time, digits=1)), ",
            "E = $(round(output.potential_energy + output.kinetic_energy, digits=2)),  ",
            "E_pot = $(round(output.potential_energy, digits=12)),  ",
            "E_pot_test = $(round(energy_no_neigh, digits=12)),  ",
            "E_kin = $(round(output.kinetic_energy, digits=2)), ",
            "kT = $(round(output.kinetic_energy * 2 / parameters.system.dims / parameters.N, digits=3)), ",
            "F₂s = $(round(output.F2s, digits=3))")
    flush(stdout)
end

"""find_inherent_structure (src/InherentStructure.jl:5-56) on the device"""
function find_inherent_structure(r_array_to_be_minimized, parameters, arrays, nl::GPUNeighborList, output;
                                 tolerance=10^-6, max_iterations=10^6, max_step_size=0.001, verbose=1)
    arrays.r_array .= r_array_to_be_minimized
    begin!(nl, arrays, parameters, output)
    it = Ref{Int64}(0)
    st = ccall((:simmd_inherent_structure, libsimmd), Cint, (Ptr{Cvoid}, Float64, Int64, Float64, Float64, Ref{Int64}),
               nl.ctx, Float64(tolerance), Int64(max_iterations), max_step_size, 0.005, it)
    from_device!(nl, arrays)
    check(st)
    verbose > 0 && println("Inherent structure found after $(it[]) iterations")
    arrays.r_array
end

# the reference's neighbour-list fields, exported from the device on access
function Base.getproperty(nl::GPUNeighborList, s::Symbol)
    if s in (:neighbor_numbers_half, :neighbor_list_half, :neighbor_numbers_full, :neighbor_list_full)
        which = s in (:neighbor_numbers_half, :neighbor_list_half) ? Int32(0) : Int32(1)
        K = getfield(nl, :dev).maxneighbours
        counts = zeros(Int64, getfield(nl, :N))
        list = zeros(Int64, K, getfield(nl, :N))
        check(ccall((:simmd_export_pairs, libsimmd), Cint, (Ptr{Cvoid}, Int32, Int64, Ptr{Int64}, Ptr{Int64}),
                    getfield(nl, :ctx), which, K, counts, list))
        return s in (:neighbor_numbers_half, :neighbor_numbers_full) ? counts : list
    end
    getfield(nl, s)
end

"""queue the copy of r, v, F into page-locked host buffers (d x N Float64
matrices registered with simmd_host_register) while later steps run"""
function gpu_dump_async(nl::GPUNeighborList, r::Matrix{Float64}, v::Matrix{Float64}, F::Matrix{Float64})
    check(ccall((:simmd_dump_async, libsimmd), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                nl.ctx, 0, pointer(r), pointer(v), pointer(F)))
end

gpu_dump_wait(nl::GPUNeighborList) = check(ccall((:simmd_dump_wait, libsimmd), Cint, (Ptr{Cvoid},), nl.ctx))

"""filtered force lists: the force pass reads the pairs within rc_ij +
inner_skin and re-filters when a particle has moved inner_skin / 2
(bit-identical results; one thread per particle); 0 turns them off"""
gpu_set_prune!(nl::GPUNeighborList, inner_skin::Real) =
    check(ccall((:simmd_set_prune, libsimmd), Cint, (Ptr{Cvoid}, Int32, Float64), nl.ctx, Int32(-1),
                Float64(inner_skin)))

"""device self-check: mismatches of the split kernels' bit-level float <->
double conversions against the hardware converter (0 expected)"""
function gpu_check_conversions(n::Integer=1 << 24, seed::Integer=1)
    bad = Ref{Int64}(-1)
    check(ccall((:simmd_check_conversions, libsimmd), Cint, (Int64, UInt64, Ref{Int64}), n, seed, bad))
    bad[]
end

devptr(x) = Ptr{Cvoid}(UInt(pointer(x)))   # a CuArray's device address (CuPtr -> UInt)

"""energy and virial of device arrays the caller owns (CuArrays from
CUDA.jl's pool), without any device allocation by libsimmd: out[1] = E_pot,
out[2] = virial, out[3] = invalid list entries skipped.  r: dims x N
Float64, D: N, counts: N Int64, list: maxK x N Int64 (the reference's
NeighborListStruct layout, 1-based), out: 3 Float64; stream: the CUstream
to run on (CUDA.stream().handle; C_NULL = the default stream).  N must be
<= SIMMD_NOALLOC_MAX_N; two such calls must not overlap on one GPU (they
share the library's fixed scratch).  Asynchronous: synchronise the stream
before reading out.  The first call on a device may load the library's
device code; make it before any stream capture."""
function gpu_energy_virial_noalloc!(out, prm::SimmdParams, r, D, counts, list, stream::Ptr{Cvoid}=C_NULL)
    prm.N <= SIMMD_NOALLOC_MAX_N || error("N beyond SIMMD_NOALLOC_MAX_N")
    maxK = Int64(size(list, 1))
    check(ccall((:simmd_energy_virial_noalloc, libsimmd), Cint,
                (Ref{SimmdParams}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int64, Ptr{Cvoid}, Ptr{Cvoid}),
                Ref(prm), devptr(r), devptr(D), devptr(counts), devptr(list), maxK, devptr(out), stream))
end

end # module
