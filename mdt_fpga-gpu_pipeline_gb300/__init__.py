"""GB300-native MDT FX correlator hot path.

The compute lives in libmdtfx.so (CUDA C++, sm_103a, C ABI declared in
include/mdt_fx.h).  This package is its thin host-side binding: it loads the
library with ctypes and exposes

* the reference's drop-in interface for this path, under the reference's
  names: PFB_Window_min4term_BH, PpS_Batch, ReorderFOutput (launched with an
  explicit grid and block as the reference client launches them,
  MDT_OneStation_client.cu:589,1083,1114), and the cuFFT / cuBLAS calls of
  the same sequence (cufftPlan1d, cufftExecC2C, cublasCgemmBatched ...),
  which resolve to this library's own kernels;
* the stage entry points and the plan API (FxPlan) of the fused pipeline.

There is no CPU fallback: if libmdtfx.so cannot be built or loaded, every
entry point raises.  Device buffers are passed as torch CUDA tensors (or raw
integer addresses); PyTorch is only used for device memory and streams.
"""
from .binding import (  # noqa: F401
    LIB_PATH, MdtError, build, lib, check, ptr, stream_handle,
    PFB_Window_min4term_BH, PpS_Batch, ReorderFOutput,
    cufftPlan1d, cufftSetStream, cufftExecC2C, cufftDestroy, cufftGetVersion,
    cublasCreate, cublasSetStream, cublasDestroy, cublasCgemmBatched,
    CUFFT_FORWARD, CUFFT_INVERSE, CUFFT_C2C, CUBLAS_OP_N, CUBLAS_OP_T, CUBLAS_OP_C,
    window_hamming_sinc, fft_c2c, xengine_f32, fengine_f32, synth_iq,
    fengine_x16, xengine_tc, x16_bytes, fengine_c64b, fx_integrate_static,
    FxPlan, FxBatch, MDT_PREC_FP32, MDT_PREC_FP16, MDT_PREC_BF16, MDT_PREC_INT8,
    fengine_q8, xengine_q8, fengine_tc, fengine_tc_q8, tc_peak_f16, fp32_peak,
    apply_gains, xengine_adjoint_f32, gain_adjoint, pfb_tap_grad,
    PacketFormat, packet_format, depacketise_seen_words, depacketise, depacketise_finish,
    STATS_FIELDS, Ingest, num_baselines, format_baselines, write_csv, write_binary,
)
from . import configs  # noqa: F401
