"""
    GBBLAS

Julia front end of libgbblas (the GB300 GEMM behind jBLAS.jl's `jmul!`).  A thin `ccall`
layer over the C ABI in `include/gbblas.h`:

    jmul!(D, A, X[, Val(...) x 5])  D = A * X, jBLAS's per-element FMA order (src/gemm.jl:244);
                                   the prefetch Val hints are accepted and unused; host `Matrix`
                                   operands go through the blocking host-buffer call
    fastmul!(D, A, X)              the small-matrix single-tile product (src/kernels.jl:202-208)
    kernel!(pD, pA, pX, Kernel{Mₖ,Pₖ,stride_AD,stride_X,N}())   D += A*X as jBLAS's pointer kernel
    initkernel!(pD, pA, pX, Kernel{...}())                        D = A*X (src/kernels.jl:212-273)
    gemm!(C, A, B)                 the same call spelled as in the task (`jmul!` semantics)
    gemm!(C, A, B, α, β; mode, slices)   BLAS-3 form; mode = :native | :ozaki | :ozaki_crt (Float64),
                                         :native | :bf16x3 | :bf16x6 (Float32)
    gemm_adjoint!(dA, dB, A, B, dC)      dA = dC*B', dB = A'*dC in one launch (Float32)
    mul!(C, A, B, α, β; mode, slices)    LinearAlgebra.mul! semantics, A and B may be
                                         transpose/adjoint views (real element types)
    enable_mul!(T)                       routes LinearAlgebra.mul! for device matrix type T here
    gemm_strided_batched!(C, A, B, α, β) C[:,:,i] = α A[:,:,i] B[:,:,i] + β C[:,:,i]
    semiring_mul!(C, A, B, semiring; accumulate)   C = [C ⊕] A ⊗ B over (min,+), (max,+),
                                         (max,min), (min,max) or (max,*) (Float64/Float32/Int32)
    ChainRulesCore.rrule(::typeof(gemm), A, B)   pullback through gemm_adjoint!
    tc_tuning, set_tc_tuning!, reset_tc_tuning!, autotune_tc!   the tensor-core tuning table

Matrices are device arrays (anything with `pointer` to CUDA device memory and a column-
major layout, e.g. CUDA.jl's `CuArray`); `stream` defaults to the task-local stream of
CUDA.jl when that package is loaded, else the legacy default stream (C_NULL).
"""
module GBBLAS

const libgbblas = get(ENV, "GBBLAS_LIB", joinpath(@__DIR__, "..", "lib", "libgbblas.so"))

const GB_OK = Cint(0)
const MODE = Dict(:native => Cint(0), :ozaki => Cint(1), :ozaki_bf16 => Cint(1), :ozaki_int8 => Cint(2),
                  :ozaki_crt => Cint(3), :bf16x3 => Cint(4), :bf16x6 => Cint(5))

struct GBError <: Exception
    status::Cint
end
Base.showerror(io::IO, e::GBError) =
    print(io, "gbblas: ", unsafe_string(ccall((:gb_status_string, libgbblas), Cstring, (Cint,), e.status)),
          " (status ", e.status, ")")

check(st::Cint) = st == GB_OK ? nothing : throw(GBError(st))

# Stream handle: CUDA.jl's current stream if the package is present, otherwise NULL.
current_stream() = isdefined(Main, :CUDA) ? Base.unsafe_convert(Ptr{Cvoid}, Main.CUDA.stream().handle) : C_NULL

ld(X::AbstractMatrix) = max(1, stride(X, 2))

# The device address of an array as a plain `Ptr` for the C ABI: CUDA.jl's `pointer` gives a
# `CuPtr`, which Julia does not convert to `Ptr`; both are 64-bit addresses, so the bits are
# reinterpreted (a plain `Ptr` passes through unchanged).
devptr(X::AbstractArray{T}) where {T} = reinterpret(Ptr{T}, pointer(X))

"""
    jmul!(D, A, X) -> D

`D = A * X` for `A` (M×N), `X` (N×P), the reference's argument order and naming (N is the
contraction dimension).  Results equal jBLAS's FMA chain bit for bit, every element
written.
"""
function jmul!(D::AbstractMatrix{Float64}, A::AbstractMatrix{Float64}, X::AbstractMatrix{Float64})
    M, N = size(A); P = size(X, 2)
    size(X, 1) == N && size(D) == (M, P) || throw(DimensionMismatch("jmul!: $(size(D)) = $(size(A)) * $(size(X))"))
    check(ccall((:gb_gemm_f64, libgbblas), Cint,
                (Cint, Cint, Int64, Int64, Int64, Cdouble, Ptr{Cdouble}, Int64, Ptr{Cdouble}, Int64, Cdouble,
                 Ptr{Cdouble}, Int64, Cint, Cint, Ptr{Cdouble}, Ptr{Cvoid}),
                0, 0, M, P, N, 1.0, devptr(A), ld(A), devptr(X), ld(X), 0.0, devptr(D), ld(D),
                MODE[:native], 0, C_NULL, current_stream()))
    D
end
function jmul!(D::AbstractMatrix{Float32}, A::AbstractMatrix{Float32}, X::AbstractMatrix{Float32})
    M, N = size(A); P = size(X, 2)
    size(X, 1) == N && size(D) == (M, P) || throw(DimensionMismatch("jmul!: $(size(D)) = $(size(A)) * $(size(X))"))
    check(ccall((:gb_gemm_f32, libgbblas), Cint,
                (Cint, Cint, Int64, Int64, Int64, Cfloat, Ptr{Cfloat}, Int64, Ptr{Cfloat}, Int64, Cfloat,
                 Ptr{Cfloat}, Int64, Ptr{Cvoid}),
                0, 0, M, P, N, 1f0, devptr(A), ld(A), devptr(X), ld(X), 0f0, devptr(D), ld(D),
                current_stream()))
    D
end

"""
    gemm!(C, A, B) -> C                      same as jmul!(C, A, B)
    gemm!(C, A, B, α, β; mode=:native, slices=0) -> C

`C = α A B + β C`.  `mode = :ozaki` (Float64) emulates FP64 on the BF16 tensor cores with
`slices` digit planes; `mode = :ozaki_crt` forms the exact product of the t-bit scaled
operands from `slices` residue products (Chinese remainder theorem; the faster mode).
`slices = 0`: the library picks the count for its normwise tolerance.
"""
gemm!(C, A, B) = jmul!(C, A, B)
function gemm!(C::AbstractMatrix{Float64}, A::AbstractMatrix{Float64}, B::AbstractMatrix{Float64}, α::Real, β::Real;
               mode::Symbol = :native, slices::Integer = 0)
    M, K = size(A); N = size(B, 2)
    size(B, 1) == K && size(C) == (M, N) || throw(DimensionMismatch("gemm!"))
    check(ccall((:gb_gemm_f64, libgbblas), Cint,
                (Cint, Cint, Int64, Int64, Int64, Cdouble, Ptr{Cdouble}, Int64, Ptr{Cdouble}, Int64, Cdouble,
                 Ptr{Cdouble}, Int64, Cint, Cint, Ptr{Cdouble}, Ptr{Cvoid}),
                0, 0, M, N, K, α, devptr(A), ld(A), devptr(B), ld(B), β, devptr(C), ld(C),
                MODE[mode], slices, C_NULL, current_stream()))
    C
end
# Float32: mode = :native (jmul!'s FMA chain, bit for bit) or :bf16x3 / :bf16x6 (BF16 term
# products on the tensor cores, gb_gemm_f32_ex).
function gemm!(C::AbstractMatrix{Float32}, A::AbstractMatrix{Float32}, B::AbstractMatrix{Float32}, α::Real, β::Real;
               mode::Symbol = :native)
    M, K = size(A); N = size(B, 2)
    size(B, 1) == K && size(C) == (M, N) || throw(DimensionMismatch("gemm!"))
    check(ccall((:gb_gemm_f32_ex, libgbblas), Cint,
                (Cint, Cint, Int64, Int64, Int64, Cfloat, Ptr{Cfloat}, Int64, Ptr{Cfloat}, Int64, Cfloat,
                 Ptr{Cfloat}, Int64, Cint, Ptr{Cvoid}),
                0, 0, M, N, K, α, devptr(A), ld(A), devptr(B), ld(B), β, devptr(C), ld(C), MODE[mode],
                current_stream()))
    C
end

# Host matrices (`Matrix`, the reference's own operands): the blocking host-buffer calls upload,
# multiply on the GPU and download before returning, with the same results.
function jmul!(D::Matrix{Float64}, A::Matrix{Float64}, X::Matrix{Float64})
    M, N = size(A); P = size(X, 2)
    size(X, 1) == N && size(D) == (M, P) || throw(DimensionMismatch("jmul!: $(size(D)) = $(size(A)) * $(size(X))"))
    check(ccall((:gb_jmul_f64_host, libgbblas), Cint,
                (Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Int64, Int64, Int64, Ptr{Cvoid}),
                D, A, X, M, N, P, current_stream()))
    D
end
function jmul!(D::Matrix{Float32}, A::Matrix{Float32}, X::Matrix{Float32})
    M, N = size(A); P = size(X, 2)
    size(X, 1) == N && size(D) == (M, P) || throw(DimensionMismatch("jmul!: $(size(D)) = $(size(A)) * $(size(X))"))
    check(ccall((:gb_jmul_f32_host, libgbblas), Cint,
                (Ptr{Cfloat}, Ptr{Cfloat}, Ptr{Cfloat}, Int64, Int64, Int64, Ptr{Cvoid}),
                D, A, X, M, N, P, current_stream()))
    D
end
function gemm!(C::Matrix{Float64}, A::Matrix{Float64}, B::Matrix{Float64}, α::Real, β::Real;
               mode::Symbol = :native, slices::Integer = 0)
    M, K = size(A); N = size(B, 2)
    size(B, 1) == K && size(C) == (M, N) || throw(DimensionMismatch("gemm!"))
    check(ccall((:gb_gemm_f64_host, libgbblas), Cint,
                (Cint, Cint, Int64, Int64, Int64, Cdouble, Ptr{Cdouble}, Int64, Ptr{Cdouble}, Int64, Cdouble,
                 Ptr{Cdouble}, Int64, Cint, Cint, Ptr{Cdouble}, Ptr{Cvoid}),
                0, 0, M, N, K, α, A, max(1, M), B, max(1, K), β, C, max(1, M), MODE[mode], slices, C_NULL,
                current_stream()))
    C
end
function gemm!(C::Matrix{Float32}, A::Matrix{Float32}, B::Matrix{Float32}, α::Real, β::Real)
    M, K = size(A); N = size(B, 2)
    size(B, 1) == K && size(C) == (M, N) || throw(DimensionMismatch("gemm!"))
    check(ccall((:gb_gemm_f32_host, libgbblas), Cint,
                (Cint, Cint, Int64, Int64, Int64, Cfloat, Ptr{Cfloat}, Int64, Ptr{Cfloat}, Int64, Cfloat,
                 Ptr{Cfloat}, Int64, Ptr{Cvoid}),
                0, 0, M, N, K, α, A, max(1, M), B, max(1, K), β, C, max(1, M), current_stream()))
    C
end

"""
    fastmul!(D, A, X) -> D

jBLAS's single-tile product of small static matrices (src/kernels.jl:202-208): per element
d = a_1 x_1, then d = fma(a_n, x_n, d) — jmul!'s chain, so the same call.
"""
fastmul!(D::AbstractMatrix{T}, A::AbstractMatrix{T}, X::AbstractMatrix{T}) where {T <: Union{Float32, Float64}} =
    jmul!(D, A, X)

# jmul!'s software-prefetch distances and cache localities (src/gemm.jl:244-246) are CPU cache
# hints; accepted for drop-in use and unused on the GPU.
jmul!(D::AbstractMatrix{T}, A::AbstractMatrix{T}, X::AbstractMatrix{T}, ::Val, hints::Val...) where {T <: Union{Float32, Float64}} =
    jmul!(D, A, X)

"""
    Kernel{Mₖ,Pₖ,stride_AD,stride_X,N}()

The micro-kernel descriptor of jBLAS's pointer kernels (src/kernel_structure.jl): an Mₖ×Pₖ tile
of D, A and D with leading dimension stride_AD, X with stride_X, contraction length N.
"""
struct Kernel{Mₖ,Pₖ,stride_AD,stride_X,N} end

for (T, f) in ((Float64, :gb_kernel_f64), (Float32, :gb_kernel_f32))
    @eval begin
        function kernel!(pD::Ptr{$T}, pA::Ptr{$T}, pX::Ptr{$T},
                         ::Kernel{Mₖ,Pₖ,stride_AD,stride_X,N}) where {Mₖ,Pₖ,stride_AD,stride_X,N}
            check(ccall(($(QuoteNode(f)), libgbblas), Cint,
                        (Ptr{$T}, Ptr{$T}, Ptr{$T}, Int64, Int64, Int64, Int64, Int64, Cint, Ptr{Cvoid}),
                        pD, pA, pX, Mₖ, Pₖ, stride_AD, stride_X, N, Cint(0), current_stream()))
            nothing
        end
        function initkernel!(pD::Ptr{$T}, pA::Ptr{$T}, pX::Ptr{$T},
                             ::Kernel{Mₖ,Pₖ,stride_AD,stride_X,N}) where {Mₖ,Pₖ,stride_AD,stride_X,N}
            check(ccall(($(QuoteNode(f)), libgbblas), Cint,
                        (Ptr{$T}, Ptr{$T}, Ptr{$T}, Int64, Int64, Int64, Int64, Int64, Cint, Ptr{Cvoid}),
                        pD, pA, pX, Mₖ, Pₖ, stride_AD, stride_X, N, Cint(1), current_stream()))
            nothing
        end
    end
end
@doc """
    kernel!(pD, pA, pX, ::Kernel{Mₖ,Pₖ,stride_AD,stride_X,N})      D += A * X

jBLAS's pointer-level micro-kernel (src/kernels.jl:212-239) on device pointers (`Ptr{T}`, e.g.
`reinterpret(Ptr{Float64}, pointer(cuarray))`): per element d = fma(a_n, x_n, d) for n = 1..N
starting from D's value, bit-identical to the reference.
""" kernel!
@doc """
    initkernel!(pD, pA, pX, ::Kernel{Mₖ,Pₖ,stride_AD,stride_X,N})  D = A * X

jBLAS's initkernel! (src/kernels.jl:240-273): d = a_1 x_1, then d = fma(a_n, x_n, d), n = 2..N.
""" initkernel!

# ------------------------------------------------------------------ mul! with transposes
import LinearAlgebra
using LinearAlgebra: Transpose, Adjoint

const Wrapped{T} = Union{Transpose{T}, Adjoint{T}}
op_flag(::AbstractMatrix) = Cint(0)
op_flag(::Wrapped{<:Real}) = Cint(1)        # a real adjoint is a transpose
storage(X::AbstractMatrix) = X
storage(X::Wrapped{<:Real}) = parent(X)

"""
    mul!(C, A, B, α=true, β=false; mode=:native, slices=0) -> C

`C = α op(A) op(B) + β C` with LinearAlgebra's argument meaning, on device matrices; `A`
and `B` may be `transpose`/`adjoint` views (passed to the library as transpose flags, the
data is not copied).  Float64 accepts `mode` (`:native`, `:ozaki`, `:ozaki_crt`), Float32
`:native`, `:bf16x3` or `:bf16x6`.
"""
function mul!(C::AbstractMatrix{Float64}, A::AbstractMatrix{Float64}, B::AbstractMatrix{Float64},
              α::Number = true, β::Number = false; mode::Symbol = :native, slices::Integer = 0)
    M, K = size(A); N = size(B, 2)
    size(B, 1) == K && size(C) == (M, N) || throw(DimensionMismatch("mul!: $(size(C)) = $(size(A)) * $(size(B))"))
    As, Bs = storage(A), storage(B)
    check(ccall((:gb_gemm_f64, libgbblas), Cint,
                (Cint, Cint, Int64, Int64, Int64, Cdouble, Ptr{Cdouble}, Int64, Ptr{Cdouble}, Int64, Cdouble,
                 Ptr{Cdouble}, Int64, Cint, Cint, Ptr{Cdouble}, Ptr{Cvoid}),
                op_flag(A), op_flag(B), M, N, K, Float64(α), devptr(As), ld(As), devptr(Bs), ld(Bs), Float64(β),
                devptr(C), ld(C), MODE[mode], slices, C_NULL, current_stream()))
    C
end
function mul!(C::AbstractMatrix{Float32}, A::AbstractMatrix{Float32}, B::AbstractMatrix{Float32},
              α::Number = true, β::Number = false; mode::Symbol = :native)
    M, K = size(A); N = size(B, 2)
    size(B, 1) == K && size(C) == (M, N) || throw(DimensionMismatch("mul!: $(size(C)) = $(size(A)) * $(size(B))"))
    As, Bs = storage(A), storage(B)
    check(ccall((:gb_gemm_f32_ex, libgbblas), Cint,
                (Cint, Cint, Int64, Int64, Int64, Cfloat, Ptr{Cfloat}, Int64, Ptr{Cfloat}, Int64, Cfloat,
                 Ptr{Cfloat}, Int64, Cint, Ptr{Cvoid}),
                op_flag(A), op_flag(B), M, N, K, Float32(α), devptr(As), ld(As), devptr(Bs), ld(Bs), Float32(β),
                devptr(C), ld(C), MODE[mode], current_stream()))
    C
end

"""
    enable_mul!(T)

Make `LinearAlgebra.mul!(C, A, B, α, β)` call this library when `C` is a `T` (a device
matrix type such as CUDA.jl's `CuMatrix{Float64}`) and `A`, `B` are `T`s or their
transpose/adjoint views.  Opt-in, so host arrays keep LinearAlgebra's own methods.
"""
function enable_mul!(::Type{T}) where {T <: AbstractMatrix}
    @eval function LinearAlgebra.mul!(C::$T, A::Union{$T, Wrapped{<:Real, <:$T}}, B::Union{$T, Wrapped{<:Real, <:$T}},
                                      α::Number, β::Number)
        GBBLAS.mul!(C, A, B, α, β)
    end
    nothing
end

for (T, f) in ((Float64, :gb_gemm_strided_batched_f64), (Float32, :gb_gemm_strided_batched_f32))
    @eval function gemm_strided_batched!(C::AbstractArray{$T,3}, A::AbstractArray{$T,3}, B::AbstractArray{$T,3},
                                         α::Number = one($T), β::Number = zero($T))
        M, K, n = size(A); N = size(B, 2)
        size(B) == (K, N, n) && size(C) == (M, N, n) || throw(DimensionMismatch("gemm_strided_batched!"))
        check(ccall(($(QuoteNode(f)), libgbblas), Cint,
                    (Int64, Int64, Int64, $T, Ptr{$T}, Int64, Int64, Ptr{$T}, Int64, Int64, $T, Ptr{$T}, Int64, Int64,
                     Int64, Ptr{Cvoid}),
                    M, N, K, $T(α), devptr(A), max(1, stride(A, 2)), stride(A, 3), devptr(B), max(1, stride(B, 2)),
                    stride(B, 3), $T(β), devptr(C), max(1, stride(C, 2)), stride(C, 3), n, current_stream()))
        C
    end
end
@doc """
    gemm_strided_batched!(C, A, B, α=1, β=0) -> C

`C[:,:,i] = α A[:,:,i] B[:,:,i] + β C[:,:,i]` for every `i`, one launch (the batch form of
jBLAS's `fastmul!`), per element jBLAS's FMA chain.  Arrays are column-major device arrays.
""" gemm_strided_batched!

const SEMIRING = Dict(:min_plus => Cint(0), :max_plus => Cint(1), :max_min => Cint(2), :min_max => Cint(3),
                     :max_times => Cint(4))

for (T, f) in ((Float64, :gb_gemm_semiring_f64), (Float32, :gb_gemm_semiring_f32), (Int32, :gb_gemm_semiring_i32))
    @eval function semiring_mul!(C::AbstractMatrix{$T}, A::AbstractMatrix{$T}, B::AbstractMatrix{$T},
                                 semiring::Symbol = :min_plus; accumulate::Bool = false)
        M, K = size(A); N = size(B, 2)
        size(B, 1) == K && size(C) == (M, N) ||
            throw(DimensionMismatch("semiring_mul!: $(size(C)) = $(size(A)) ⊗ $(size(B))"))
        As, Bs = storage(A), storage(B)
        check(ccall(($(QuoteNode(f)), libgbblas), Cint,
                    (Cint, Cint, Cint, Int64, Int64, Int64, Ptr{$T}, Int64, Ptr{$T}, Int64, Cint, Ptr{$T}, Int64,
                     Ptr{Cvoid}),
                    SEMIRING[semiring], op_flag(A), op_flag(B), M, N, K, devptr(As), ld(As), devptr(Bs), ld(Bs),
                    Cint(accumulate), devptr(C), ld(C), current_stream()))
        C
    end
end
@doc """
    semiring_mul!(C, A, B, semiring=:min_plus; accumulate=false) -> C

`C[i,j] = ⊕_k A[i,k] ⊗ B[k,j]` (or `C[i,j] ⊕ ...` with `accumulate`) over the semiring
`semiring` ∈ `:min_plus`, `:max_plus`, `:max_min`, `:min_max`, `:max_times` (⊕ first), the
custom-number-type use jBLAS gives for its `Vec` fallback ("so it works with min-plus
algebra", src/jBLAS.jl:10).  `A` and `B` may be transpose/adjoint views.  Floating point: ⊕
ignores NaN operands and a zero result is +0.0; Int32 + and * wrap.
""" semiring_mul!

"""
    gemm_adjoint!(dA, dB, A, B, dC) -> (dA, dB)

`dA = dC * B'` and `dB = A' * dC` (Float32) in one tensor-core launch, 3xBF16 split with
FP32 accumulation.
"""
function gemm_adjoint!(dA::AbstractMatrix{Float32}, dB::AbstractMatrix{Float32}, A::AbstractMatrix{Float32},
                       B::AbstractMatrix{Float32}, dC::AbstractMatrix{Float32})
    M, K = size(A); N = size(B, 2)
    check(ccall((:gb_gemm_adjoint_f32, libgbblas), Cint,
                (Int64, Int64, Int64, Ptr{Cfloat}, Int64, Ptr{Cfloat}, Int64, Ptr{Cfloat}, Int64, Ptr{Cfloat}, Int64,
                 Ptr{Cfloat}, Int64, Ptr{Cvoid}),
                M, N, K, devptr(A), ld(A), devptr(B), ld(B), devptr(dC), ld(dC), devptr(dA), ld(dA),
                devptr(dB), ld(dB), current_stream()))
    dA, dB
end

"""
    gemm(A, B)

Allocating product for use with automatic differentiation: the `rrule` below returns
the pullback computed by `gemm_adjoint!` (Float32) or two Ozaki products (Float64).
"""
gemm(A::AbstractMatrix, B::AbstractMatrix) = jmul!(similar(A, size(A, 1), size(B, 2)), A, B)

# ------------------------------------------------------------------ tensor-core tuning
"""
    TcTuning(engine, band, tma_store, panels)

`gb_tc_tuning_t`: the launch configuration of the tensor-core engine for one kind of product
and output-size class (engine 1 = one CTA per 128 x 256 tile, 2 = a CTA pair per 256 x 256
tile; band = tile rows per L2 band; tma_store = TMA stores of FP32 outputs; panels = CRT
blocks of C) — the measured counterpart of jBLAS's `pick_kernel_size` and `BLASOptions`
(src/kernel_structure.jl:76-99, src/blas_options.jl:2-7).
"""
struct TcTuning
    engine::Int32
    band::Int32
    tma_store::Int32
    panels::Int32
end

const TC_KIND = Dict(:ozaki_slices => Cint(0), :ozaki_crt => Cint(1), :f32 => Cint(2), :adjoint => Cint(3))

"Size class of an M x N output for the tuning table (by max(M, N): 0 up to 2048, 1 up to 8192, 2 beyond)."
tc_size_class(M::Integer, N::Integer) = Int(ccall((:gb_tc_size_class, libgbblas), Cint, (Int64, Int64), M, N))

"The tuning that calls of `kind` (:ozaki_slices, :ozaki_crt, :f32, :adjoint) in `size_class` use."
function tc_tuning(kind::Symbol, size_class::Integer)
    r = Ref{TcTuning}()
    check(ccall((:gb_get_tc_tuning, libgbblas), Cint, (Cint, Cint, Ptr{TcTuning}), TC_KIND[kind], size_class, r))
    r[]
end

"Installs `t` for later calls of `kind` in `size_class`; `reset_tc_tuning!` restores the default."
set_tc_tuning!(kind::Symbol, size_class::Integer, t::TcTuning) =
    check(ccall((:gb_set_tc_tuning, libgbblas), Cint, (Cint, Cint, Ref{TcTuning}), TC_KIND[kind], size_class, t))
reset_tc_tuning!(kind::Symbol, size_class::Integer) =
    check(ccall((:gb_set_tc_tuning, libgbblas), Cint, (Cint, Cint, Ptr{TcTuning}), TC_KIND[kind], size_class, C_NULL))

"""
    autotune_tc!(kind, M, N, K; reps = 3, install = true) -> (TcTuning, ms)

Times the candidate configurations of `kind` on seeded M x N x K operands on the device
(`gb_autotune_tc`) and, with `install`, sets the fastest for that size class.  Persist the
result with the standard library's `Serialization` (or any format) and install it in a later
session with `set_tc_tuning!`.
"""
function autotune_tc!(kind::Symbol, M::Integer, N::Integer, K::Integer; reps::Integer = 3, install::Bool = true)
    t = Ref{TcTuning}()
    ms = Ref{Cfloat}(0)
    check(ccall((:gb_autotune_tc, libgbblas), Cint,
                (Cint, Int64, Int64, Int64, Cint, Ptr{TcTuning}, Ptr{Cfloat}, Ptr{Cvoid}),
                TC_KIND[kind], M, N, K, reps, t, ms, current_stream()))
    install && set_tc_tuning!(kind, tc_size_class(M, N), t[])
    t[], Float64(ms[])
end

"""
    crt_blocks(M, N, panels, sms; host_copies = false) -> (rows, cols)

Row and column boundaries of the blocks of C an Ozaki CRT call cuts an M x N output into
(`gb_crt_blocks`), for the tuning's `panels`, a device of `sms` SMs and, with `host_copies`, a
host-buffer call on a pinned C.  No GPU work.
"""
function crt_blocks(M::Integer, N::Integer, panels::Integer, sms::Integer; host_copies::Bool = false)
    rows = zeros(Int64, 3)
    cols = zeros(Int64, 5)
    nr = Ref{Cint}(0)
    nc = Ref{Cint}(0)
    check(ccall((:gb_crt_blocks, libgbblas), Cint,
                (Int64, Int64, Cint, Cint, Cint, Ptr{Int64}, Ref{Cint}, Ptr{Int64}, Ref{Cint}),
                M, N, panels, sms, host_copies ? 1 : 0, rows, nr, cols, nc))
    rows[1:nr[]+1], cols[1:nc[]+1]
end

# ChainRulesCore is optional: the rrule is defined when the package is available.
if Base.find_package("ChainRulesCore") !== nothing
    import ChainRulesCore
    function ChainRulesCore.rrule(::typeof(gemm), A::AbstractMatrix{Float32}, B::AbstractMatrix{Float32})
        C = gemm(A, B)
        function gemm_pullback(ΔC)
            dC = convert(typeof(C), ChainRulesCore.unthunk(ΔC))
            dA, dB = gemm_adjoint!(similar(A), similar(B), A, B, dC)
            return ChainRulesCore.NoTangent(), dA, dB
        end
        return C, gemm_pullback
    end
    function ChainRulesCore.rrule(::typeof(gemm), A::AbstractMatrix{Float64}, B::AbstractMatrix{Float64})
        C = gemm(A, B)
        function gemm_pullback(ΔC)
            dC = convert(typeof(C), ChainRulesCore.unthunk(ΔC))
            # transposes as views: the library reads them through its transpose flags, no copies
            dA = mul!(similar(A), dC, transpose(B), 1.0, 0.0; mode = :ozaki_crt)
            dB = mul!(similar(B), transpose(A), dC, 1.0, 0.0; mode = :ozaki_crt)
            return ChainRulesCore.NoTangent(), dA, dB
        end
        return C, gemm_pullback
    end
end

end # module
