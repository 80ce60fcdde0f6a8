# GB300Ext: the explicit MPM time loop of ElastoPlasm.jl on one GB300 through libepgpu.so.
#
# The binding an ElastoPlasm.jl maintainer would add beside ext/CUDAExt.jl.  It keeps the
# reference's `Point`/`Mesh` structs (src/boot/needs/types.jl:38-168) and its workflow
# (src/home/program/workflow/worflow.jl:23-141), and hands the loop over one checkpoint list to
# `epgpu_run_checkpoints` (include/epgpu.h); `savlot` runs from the library's checkpoint callback.
# The library never sees a Julia type: only pointers to the column-major arrays, which the library
# transposes to its own device layout on upload and back on download.
#
# Use (the cfg switch of `elastoplasm`, worflow.jl:113-141):
#     cfg.instr[:gpu] = (; precision = "fp64" | "mixed" | "mixed_df", deterministic = false)
#     out = GB300Ext.elastoplasm(ic, cfg; mode = "all-in-one")
# The library path comes from ENV["EPGPU_LIB"] (default: the in-tree build,
# elastoplasm.jl_gb300/lib/libepgpu.so).
#
# Julia is not available where this repository is built and tested; the C side of every call here
# is exercised through the same entry points by the Python host (tests/*.py).
module GB300Ext

using ElastoPlasm: Point, Mesh, savlot, elastoplasm_log, exit_log, save_plot

const LIB = get(ENV, "EPGPU_LIB", joinpath(@__DIR__, "..", "lib", "libepgpu.so"))

# ---- ABI mirrors (field order and C types as include/epgpu.h) ---------------------------------
struct EpCfg
    dim::Int32; basis::Int32; how::Int32; ghost::Int32; deform::Int32; trsfr::Int32
    C_pf::Float64
    musl::Int32; locking::Int32
    damping::Float64
    constitutive::Int32; nonloc::Int32
    nonloc_ls::Float64
    precision::Int32; jaumann::Int32; deterministic::Int32
end

struct EpCmpr
    E::Float64; nu::Float64; Kc::Float64; Gc::Float64
    Del::NTuple{36,Float64}
    Hp::Float64; c0::Float64; cr::Float64; phi0::Float64; phir::Float64; rho0::Float64; c::Float64
end

struct EpMeshView
    dim::Int64; nel::NTuple{4,Int64}; nno::NTuple{4,Int64}; nn::Int64
    h::NTuple{3,Float64}; x0::NTuple{3,Float64}
    x::Ptr{Float64}; xB::Ptr{Float64}; bcs::Ptr{UInt8}; e2n::Ptr{Int64}
end

struct EpMptsView
    ndim::Int64; nmp::Int64
    vmax::Ptr{Float64}; x::Ptr{Float64}; l0::Ptr{Float64}; l::Ptr{Float64}
    n0::Ptr{Float64}; n::Ptr{Float64}; Omega0::Ptr{Float64}; Omega::Ptr{Float64}; dJ::Ptr{Float64}; J::Ptr{Float64}
    u::Ptr{Float64}; v::Ptr{Float64}; p::Ptr{Float64}
    rho0::Ptr{Float64}; rho::Ptr{Float64}; c0::Ptr{Float64}; cr::Ptr{Float64}; phi::Ptr{Float64}; dlam::Ptr{Float64}
    epII::Ptr{Float64}; epV::Ptr{Float64}; sig::Ptr{Float64}; tau::Ptr{Float64}
    dvij::Ptr{Float64}; duij::Ptr{Float64}; dFij::Ptr{Float64}; Fij::Ptr{Float64}; bij::Ptr{Float64}
    eij::Ptr{Float64}; wij::Ptr{Float64}; sJij::Ptr{Float64}
    p2e::Ptr{Int64}; p2n::Ptr{Int64}
    Bij::Ptr{Float64}; Dij::Ptr{Float64}
end

# ---- switch tables (require.jl:34-88 spellings -> the header's enums) --------------------------
const BASIS = Dict("bsmpm" => 0, "gimpm" => 1, "smpm" => 2)
const HOW = Dict{Any,Int}(nothing => 0, "undeformed" => 1, "detFij" => 2, "Fii" => 3, "Uii" => 4,
                          "detΔFij" => 5, "ΔFii" => 6, "ΔUii" => 7)
const DEFORM = Dict("finite" => 0, "infinitesimal" => 1)
const TRSFR = Dict("std" => 0, "tpic" => 1, "apic" => 2)
const CONS = Dict("DP" => 0, "J2" => 1, "MC" => 2, "camC" => 3)
const PREC = Dict("fp64" => 0, "mixed" => 1, "mixed_df" => 2)

function switch(tab, key, what)
    haskey(tab, key) || throw(ArgumentError("unsupported $(what): $(key)"))
    return Int32(tab[key])
end

function ep_cfg(mesh::Mesh, instr)
    gpu = get(instr, :gpu, (;))
    EpCfg(Int32(mesh.dim), switch(BASIS, instr[:basis][:which], "basis"),
          switch(HOW, get(instr[:basis], :how, nothing), "basis.how"), Int32(instr[:basis][:ghost]),
          switch(DEFORM, instr[:fwrk][:deform], "fwrk.deform"), switch(TRSFR, instr[:fwrk][:trsfr], "fwrk.trsfr"),
          Float64(instr[:fwrk][:C_pf]), Int32(instr[:fwrk][:musl]), Int32(instr[:fwrk][:locking]),
          Float64(instr[:fwrk][:damping]), switch(CONS, instr[:plast][:constitutive], "plast.constitutive"),
          Int32(instr[:nonloc][:status]), Float64(instr[:nonloc][:ls]),
          switch(PREC, get(gpu, :precision, "fp64"), "gpu.precision"), Int32(0),
          Int32(get(gpu, :deterministic, false)))
end

function ep_cmpr(cmpr)
    del = zeros(Float64, 36)
    ns = size(cmpr.Del, 1)
    del[1:ns*ns] .= vec(cmpr.Del)                     # column-major nstr x nstr
    EpCmpr(cmpr.E, cmpr.ν, cmpr.Kc, cmpr.Gc, Tuple(del), cmpr.Hp, cmpr.c0, cmpr.cr, cmpr.ϕ0, cmpr.ϕr,
           cmpr.ρ0, cmpr.c)
end

pad(v, n, z) = ntuple(i -> i <= length(v) ? v[i] : z, n)

ep_mesh(mesh::Mesh) = EpMeshView(Int64(mesh.dim), pad(Int64.(mesh.nel), 4, 0), pad(Int64.(mesh.nno), 4, 0),
                                 Int64(mesh.nn), pad(Float64.(mesh.h), 3, 0.0), pad(Float64.(mesh.x₀), 3, 0.0),
                                 pointer(mesh.x), pointer(mesh.xB),
                                 Ptr{UInt8}(pointer(mesh.bcs.status)), pointer(mesh.e2n))

ep_mpts(m::Point) = EpMptsView(m.ndim, m.nmp, pointer(m.vmax), pointer(m.x), pointer(m.ℓ₀), pointer(m.ℓ),
    pointer(m.n₀), pointer(m.n), pointer(m.Ω₀), pointer(m.Ω), pointer(m.ΔJ), pointer(m.J),
    pointer(m.s.u), pointer(m.s.v), pointer(m.s.p), pointer(m.s.ρ₀), pointer(m.s.ρ), pointer(m.s.c₀),
    pointer(m.s.cᵣ), pointer(m.s.ϕ), pointer(m.s.Δλ), pointer(m.s.ϵpII), pointer(m.s.ϵpV),
    pointer(m.s.σᵢ), pointer(m.s.τᵢ), pointer(m.s.∇vᵢⱼ), pointer(m.s.∇uᵢⱼ), pointer(m.s.ΔFᵢⱼ),
    pointer(m.s.Fᵢⱼ), pointer(m.s.bᵢⱼ), pointer(m.s.ϵᵢⱼ), pointer(m.s.ωᵢⱼ), pointer(m.s.σJᵢⱼ),
    pointer(m.p2e), pointer(m.p2n), pointer(m.Bᵢⱼ), pointer(m.Dᵢⱼ))

# ---- calls --------------------------------------------------------------------------------------
last_error(h) = unsafe_string(ccall((:epgpu_last_error, LIB), Cstring, (Ptr{Cvoid},), h))
check(st, h) = st == 0 || error("libepgpu: status $(st): $(last_error(h))")

mutable struct Session
    h::Ptr{Cvoid}
    mpts::Point
    mesh::Mesh
    instr::Any
    view::Base.RefValue{EpMptsView}
    failure::Any
end

# savlot at every checkpoint (worflow.jl:41,87): download the Point, then the reference's plotting.
function on_checkpoint(h::Ptr{Cvoid}, k::Int32, t::Float64, user::Ptr{Cvoid})::Int32
    s = unsafe_pointer_to_objref(user)::Session
    try
        check(ccall((:epgpu_download, LIB), Cint, (Ptr{Cvoid}, Ref{EpMptsView}), h, s.view), h)
        savlot(s.mpts, s.mesh, t, s.instr)
        return Int32(0)
    catch err                     # no Julia exception may unwind through the C library
        s.failure = err
        return Int32(1)
    end
end

function phase!(s::Session, phase::Integer, time, t_end)
    checks = sort(collect(time.t[1]:s.instr[:plot][:freq]:t_end))      # worflow.jl:24,69
    t = Ref(Float64(time.t[1]))
    cb = @cfunction(on_checkpoint, Int32, (Ptr{Cvoid}, Int32, Float64, Ptr{Cvoid}))
    GC.@preserve s checks begin
        st = ccall((:epgpu_run_checkpoints, LIB), Cint,
                   (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32, Float64, Ref{Float64}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}),
                   s.h, Int32(phase), checks, Int32(length(checks)), Float64(time.tg), t, cb,
                   pointer_from_objref(s), C_NULL)
    end
    s.failure === nothing || throw(s.failure)
    check(st, s.h)
    time.t[1] = t[]
    return nothing
end

"""
    elastoplasm(ic, cfg; mode="elastodynamic")

`ElastoPlasm.elastoplasm` (worflow.jl:113-141) with the time loop on the GPU: the Point is uploaded
once, each phase walks its checkpoint list in one `epgpu_run_checkpoints` call, and the Point is
downloaded at every checkpoint (for `savlot`) and at the end.
"""
function elastoplasm(ic::NamedTuple, cfg::NamedTuple; mode::String = "elastodynamic")
    mesh, mpts, cmpr = ic[:mesh], ic[:mpts], ic[:cmpr]
    time = ic[:time]
    instr, paths, misc = cfg[:instr], cfg[:paths], cfg[:misc]
    mode in ("elastodynamic", "elastoplastic", "all-in-one") ||
        (@error "Invalid workflow: $(mode). Choose 'elastodynamic', 'elastoplastic' or 'all-in-one'."; return false)
    @info elastoplasm_log(instr; msg = mode)
    c, cm, mv = ep_cfg(mesh, instr), ep_cmpr(cmpr), ep_mesh(mesh)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve mesh mpts begin
        check(ccall((:epgpu_create, LIB), Cint,
                    (Ref{EpCfg}, Ref{EpCmpr}, Ref{EpMeshView}, Int64, Ref{Ptr{Cvoid}}),
                    c, cm, mv, Int64(mpts.nmp), h), C_NULL)
        s = Session(h[], mpts, mesh, instr, Ref(ep_mpts(mpts)), nothing)
        try
            check(ccall((:epgpu_upload, LIB), Cint, (Ptr{Cvoid}, Ref{EpMptsView}), s.h, s.view), s.h)
            mode != "elastoplastic" && phase!(s, 0, time, time.te)        # elastodynamic!
            mode != "elastodynamic" && phase!(s, 1, time, time.t[2])      # elastoplastic!
            check(ccall((:epgpu_download, LIB), Cint, (Ptr{Cvoid}, Ref{EpMptsView}), s.h, s.view), s.h)
        finally
            ccall((:epgpu_destroy, LIB), Cint, (Ptr{Cvoid},), s.h)
        end
    end
    if instr[:plot][:status]
        save_plot((; file = joinpath(paths[:plot], "$(misc[:file]).png")))
    end
    exit_log("(✓) Done! exiting...\n")
    return (; ic, cfg)
end

end # module
