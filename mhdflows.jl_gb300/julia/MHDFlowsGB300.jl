# Julia binding of libmhdgb (include/mhdgb.h) for MHDFlows.jl.
#
# Provides a time stepper that plugs into MHDFlows the same way HM89TimeStepper does
# (src/timestepper/HM89.jl:6-31 of MHDFlows.jl): a struct <: FourierFlows.AbstractTimeStepper
# plus a stepforward! method, selected in MHDFLowsProblem (src/Problems.jl:124-129) by
# stepper = "GB300RK4" or "GB300LSRK4".  prob.sol stays authoritative: every stepforward! pushes
# the caller's array into the library, steps, and writes the result back into it, so
# Diagnostic, DivVCorrection!, savefile and user code that read or edit prob.sol between steps
# see and change the current state.  For a CuArray (Problem(GPU(); ...)) the push and the
# write-back are device-to-device kernels ordered on the array's stream.
#
# Not exercised in this repository's test suite (no Julia toolchain is available here); the
# same C ABI is exercised from Python through ctypes with identical signatures.
module MHDFlowsGB300

using FourierFlows
using CUDA
import FourierFlows: stepforward!

export GB300TimeStepper, gb300_updatevars!, sync_sol!, push_sol!, gb300_diagnostics, gb300_autotune!, gb300_set_cfl!,
       gb300_SetUpFk!, gb300_set_vp!, gb300_DivVCorrection!, gb300_DivBCorrection!, gb300_div_correction!,
       gb300_record_diagnostics!, gb300_diagnostic_history, MhdServerParams, MhdRequest, GB300Server,
       gb300_submit!, gb300_tick!, gb300_poll, gb300_result

const libmhdgb = get(ENV, "MHDGB_LIB", joinpath(@__DIR__, "..", "lib", "libmhdgb.so"))

struct MhdParams
  n::Cint
  L::Cdouble
  nu::Cdouble
  eta::Cdouble
  nnu::Cint
  neta::Cint
  dt::Cdouble
  scheme::Cint
  precision::Cint
  device::Cint
  hydro_only::Cint
  vp::Cint
end

check(rc) = rc == 0 ? nothing : error(unsafe_string(ccall((:mhd_last_error, libmhdgb), Cstring, ())))

mutable struct GB300TimeStepper{T} <: FourierFlows.AbstractTimeStepper{T}
  handle::Ptr{Cvoid}
  n::Int
  cfl::Bool   # the on-device getCFL! owns dt and t (gb300_set_cfl!)
end

function GB300TimeStepper(grid, params, dt; scheme::Symbol = :RK4, device::Integer = 0,
                          B_field::Bool = true, precision::Symbol = :FP32, VP_method::Bool = false)
  grid.nx == grid.ny == grid.nz || error("GB300TimeStepper needs a cubic grid")
  prec = precision == :FP32 ? 0 : precision == :SPLIT_FP16 ? 1 : precision == :SPLIT_BF16 ? 2 :
         error("precision must be :FP32, :SPLIT_FP16 or :SPLIT_BF16")
  eta = B_field ? params.η : 0.0
  neta = B_field ? params.nη : 0
  p = MhdParams(grid.nx, grid.Lx, params.ν, eta, params.nν, neta, dt,
                scheme == :RK4 ? 0 : 1, prec, device, B_field ? 0 : 1, VP_method ? 1 : 0)
  h = Ref{Ptr{Cvoid}}(C_NULL)
  check(ccall((:mhd_create, libmhdgb), Cint, (Ref{MhdParams}, Ref{Ptr{Cvoid}}), p, h))
  ts = GB300TimeStepper{Array{ComplexF32,4}}(h[], grid.nx, false)
  finalizer(t -> ccall((:mhd_destroy, libmhdgb), Cint, (Ptr{Cvoid},), t.handle), ts)
  return ts
end

# prob.sol ((nkr, n, n, 6) ComplexF32) <-> library state.  A CuArray moves by a device kernel on
# the task's stream (mhd_set_state_device / mhd_get_state_device); a host Array by copies.
devptr(a::CuArray) = Ptr{Cvoid}(UInt(pointer(a)))
streamptr() = reinterpret(Ptr{Cvoid}, CUDA.stream().handle)

push_sol!(ts::GB300TimeStepper, sol::CuArray) =
  check(ccall((:mhd_set_state_device, libmhdgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
              ts.handle, devptr(sol), streamptr()))
push_sol!(ts::GB300TimeStepper, sol::Array{ComplexF32}) =
  check(ccall((:mhd_set_state, libmhdgb), Cint, (Ptr{Cvoid}, Ptr{ComplexF32}), ts.handle, sol))
push_sol!(ts::GB300TimeStepper, sol) = push_sol!(ts, Array{ComplexF32}(sol))

sync_sol!(sol::CuArray, ts::GB300TimeStepper) =
  check(ccall((:mhd_get_state_device, libmhdgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
              ts.handle, devptr(sol), streamptr()))
sync_sol!(sol::Array{ComplexF32}, ts::GB300TimeStepper) =
  check(ccall((:mhd_get_state, libmhdgb), Cint, (Ptr{Cvoid}, Ptr{ComplexF32}), ts.handle, sol))
function sync_sol!(sol, ts::GB300TimeStepper)
  host = Array{ComplexF32}(undef, size(sol))
  sync_sol!(host, ts)
  copyto!(sol, host)
  return nothing
end

# stepforward!(sol, clock, ts, equation, vars, params, grid): one step of the library on the
# caller's current sol, written back into sol.  With a fixed step the clock is the caller's (it
# is handed to the library first, so edits of clock.t / clock.dt take effect); with the
# on-device getCFL! (gb300_set_cfl!) the library owns dt and t and the clock is read back.
function stepforward!(sol, clock, ts::GB300TimeStepper, equation, vars, params, grid)
  if !ts.cfl
    check(ccall((:mhd_set_clock, libmhdgb), Cint, (Ptr{Cvoid}, Cdouble, Clonglong, Cdouble),
                ts.handle, clock.t, clock.step, clock.dt))
  end
  push_sol!(ts, sol)
  check(ccall((:mhd_step, libmhdgb), Cint, (Ptr{Cvoid}, Cint), ts.handle, 1))
  sync_sol!(sol, ts)
  if ts.cfl
    t, step, dt = Ref{Cdouble}(0), Ref{Clonglong}(0), Ref{Cdouble}(0)
    check(ccall((:mhd_get_clock, libmhdgb), Cint, (Ptr{Cvoid}, Ref{Cdouble}, Ref{Clonglong}, Ref{Cdouble}),
                ts.handle, t, step, dt))
    clock.t, clock.dt = t[], dt[]
  else
    clock.t += clock.dt
  end
  clock.step += 1
  return nothing
end

# getCFL! of TimeIntegrator! (src/integrator.jl:54-58, 158-198) on the device: every step ends
# with dt = min(CFL_Coef dx / max(|u|, |B|), t_diff) and the library advances t.
function gb300_set_cfl!(ts::GB300TimeStepper, enable::Bool; CFL_Coef = 0.25)
  check(ccall((:mhd_set_cfl, libmhdgb), Cint, (Ptr{Cvoid}, Cint, Cdouble), ts.handle, enable ? 1 : 0, CFL_Coef))
  ts.cfl = enable
  return nothing
end

# updatevars!(prob): vars.ux..bz <- irfft(sol) of the current state
function gb300_updatevars!(prob)
  ts = prob.timestepper
  names = hasproperty(prob.vars, :bx) ? (:ux, :uy, :uz, :bx, :by, :bz) : (:ux, :uy, :uz)
  for (f, name) in enumerate(names)
    host = Array{Float32}(undef, ts.n, ts.n, ts.n)
    check(ccall((:mhd_get_physical, libmhdgb), Cint, (Ptr{Cvoid}, Cint, Ptr{Float32}), ts.handle, f - 1, host))
    copyto!(getfield(prob.vars, name), host)
  end
  return nothing
end

# E_u, E_B, H_c, max|k.u|, max|k.B|, max|div B|, non-finite count, t
function gb300_diagnostics(ts::GB300TimeStepper)
  out = zeros(Float64, 8)
  rc = ccall((:mhd_diagnostics, libmhdgb), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cint), ts.handle, out, 8)
  check(rc)
  return out
end

# Kernel variants: time the candidates of each FFT pass once for this device and grid size (the
# choice is cached per process and in the tuning file; flags: 1 = force, 2 = no file).
gb300_autotune!(ts::GB300TimeStepper; force::Bool = false) =
  check(ccall((:mhd_autotune, libmhdgb), Cint, (Ptr{Cvoid}, Cint), ts.handle, force ? 1 : 0))

# SetUpFk!(prob; kf, P, σ, b) + the A99ForceDriving! calcF! hook (src/pgen/A99ForceDriving_GPU.jl):
# P = 0 turns the forcing off; the random numbers come from a generator keyed by `seed`.
gb300_SetUpFk!(ts::GB300TimeStepper; kf = 2.0, P = 1.0, σ = 1.0, b = 1.0, seed::Integer = 0) =
  check(ccall((:mhd_set_forcing, libmhdgb), Cint,
              (Ptr{Cvoid}, Cdouble, Cdouble, Cdouble, Cdouble, Culonglong), ts.handle, P, kf, σ, b, seed))

# Volume penalisation (VP_method = true): the library's copy of params.χ, params.U₀x..U₀z and
# params.B₀x..B₀z (src/Structure/datastructure.jl:79-95).  Call after filling them, and again
# whenever they change; U₀ / B₀ = nothing means zero walls.
function gb300_set_vp!(ts::GB300TimeStepper, χ; U₀ = nothing, B₀ = nothing)
  walls(t) = t === nothing ? C_NULL : vcat(vec(Array{Float32}(t[1])), vec(Array{Float32}(t[2])), vec(Array{Float32}(t[3])))
  u, b = walls(U₀), walls(B₀)
  GC.@preserve u b begin
    check(ccall((:mhd_set_vp, libmhdgb), Cint, (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}),
                ts.handle, Array{Float32}(χ), u === C_NULL ? C_NULL : pointer(u), b === C_NULL ? C_NULL : pointer(b)))
  end
end
gb300_set_vp!(prob) = gb300_set_vp!(prob.timestepper, prob.params.χ;
                                    U₀ = (prob.params.U₀x, prob.params.U₀y, prob.params.U₀z),
                                    B₀ = hasproperty(prob.params, :B₀x) ?
                                         (prob.params.B₀x, prob.params.B₀y, prob.params.B₀z) : nothing)

# DivVCorrection!(prob) / DivBCorrection!(prob) (src/Solver/VPSolver.jl:60-138) on the device state
gb300_DivVCorrection!(ts::GB300TimeStepper) =
  check(ccall((:mhd_div_correct, libmhdgb), Cint, (Ptr{Cvoid}, Cint), ts.handle, 1))
gb300_DivBCorrection!(ts::GB300TimeStepper) =
  check(ccall((:mhd_div_correct, libmhdgb), Cint, (Ptr{Cvoid}, Cint), ts.handle, 2))

# Per-step corrections inside the library, as TimeIntegrator! does with VP after every
# stepforward! (src/integrator.jl:118-122); a TimeIntegrator! that already calls
# DivVCorrection! / DivBCorrection! itself leaves this off.
gb300_div_correction!(ts::GB300TimeStepper, on::Bool) =
  check(ccall((:mhd_set_div_correction, libmhdgb), Cint, (Ptr{Cvoid}, Cint), ts.handle, on ? 1 : 0))

# increment!(diags) on the device: every `freq` steps the spectral diagnostics are written to a
# device history of `capacity` samples, with no host synchronisation in the stepping loop.
gb300_record_diagnostics!(ts::GB300TimeStepper, freq::Integer; capacity::Integer = 1024) =
  check(ccall((:mhd_set_diag_history, libmhdgb), Cint, (Ptr{Cvoid}, Cint, Cint), ts.handle, freq, capacity))

# (samples × 8) Float64: step, t, E_u, E_B, H_c, max|k·u|, max|k·B|, non-finite count
function gb300_diagnostic_history(ts::GB300TimeStepper)
  n = Ref{Cint}(0)
  check(ccall((:mhd_get_diag_history, libmhdgb), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Ref{Cint}),
              ts.handle, 0, C_NULL, 0, n))
  out = zeros(Float64, 8, max(n[], 1))
  check(ccall((:mhd_get_diag_history, libmhdgb), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Ref{Cint}),
              ts.handle, 0, out, n[], n))
  return permutedims(out[:, 1:n[]])
end

# Serving scheduler (mhd_server_*): continuous batching of independent solves on one GPU.
struct MhdServerParams
  budget_bytes::Cdouble
  steps_per_tick::Cint
  scheme::Cint
  device::Cint
  keep_states::Cint
  capacity::NTuple{8,Cint}
end

struct MhdRequest
  n::Cint
  L::Cdouble
  nu::Cdouble
  eta::Cdouble
  dt::Cdouble
  steps::Clonglong
  sol::Ptr{ComplexF32}
end

mutable struct GB300Server
  handle::Ptr{Cvoid}
end

function GB300Server(; budget_bytes = 150e9, steps_per_tick = 8, scheme::Symbol = :RK4, device = 0,
                     keep_states::Bool = false)
  p = MhdServerParams(budget_bytes, steps_per_tick, scheme == :RK4 ? 0 : 1, device, keep_states ? 1 : 0,
                      ntuple(_ -> Cint(0), 8))
  h = Ref{Ptr{Cvoid}}(C_NULL)
  check(ccall((:mhd_server_create, libmhdgb), Cint, (Ref{MhdServerParams}, Ref{Ptr{Cvoid}}), p, h))
  s = GB300Server(h[])
  finalizer(x -> ccall((:mhd_server_destroy, libmhdgb), Cint, (Ptr{Cvoid},), x.handle), s)
  return s
end

# sol: (nkr, n, n, 6) ComplexF32 initial state (copied at submit); returns the request id
function gb300_submit!(s::GB300Server, n, L, ν, η, steps, sol; dt = 0.0)
  rid = Ref{Clonglong}(0)
  GC.@preserve sol begin
    r = MhdRequest(n, L, ν, η, dt, steps, pointer(sol))
    check(ccall((:mhd_server_submit, libmhdgb), Cint, (Ptr{Cvoid}, Ref{MhdRequest}, Ref{Clonglong}), s.handle, r, rid))
  end
  return rid[]
end

function gb300_tick!(s::GB300Server)
  a, q = Ref{Cint}(0), Ref{Cint}(0)
  check(ccall((:mhd_server_tick, libmhdgb), Cint, (Ptr{Cvoid}, Ref{Cint}, Ref{Cint}), s.handle, a, q))
  return a[], q[]
end

const REQ_STATUS = (:queued, :active, :done, :failed, :rejected, :cancelled)
function gb300_poll(s::GB300Server, rid)
  st, done = Ref{Cint}(0), Ref{Clonglong}(0)
  check(ccall((:mhd_server_poll, libmhdgb), Cint, (Ptr{Cvoid}, Clonglong, Ref{Cint}, Ref{Clonglong}), s.handle, rid, st, done))
  return REQ_STATUS[st[] + 1], done[]
end

# diagnostics (8 values as gb300_diagnostics) of a finished request
function gb300_result(s::GB300Server, rid)
  d = zeros(Float64, 8)
  check(ccall((:mhd_server_result, libmhdgb), Cint, (Ptr{Cvoid}, Clonglong, Ptr{Cdouble}, Ptr{Cvoid}),
              s.handle, rid, d, C_NULL))
  return d
end

end # module
