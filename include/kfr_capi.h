/*
 * kfr_capi.h: C ABI of the GB300 DFT library, a drop-in for KFR 7.0.1's C API (include/kfr/capi.h).
 *
 * Every declaration in the first part has the same name, argument types, argument meaning and error
 * behaviour as the reference entry point cited beside it, so a program (or a cgo / ctypes / JNI binding)
 * built against the reference header links and runs against libkfr_capi.so from this repository:
 *   - plans are opaque heap objects owned by the caller and freed with *_delete_plan (NULL allowed);
 *   - no exception crosses the ABI: failures return NULL / 0 and leave a message for kfr_last_error();
 *   - inverse transforms are unscaled; real plans use the CCs or Perm packing.
 *
 * What is different, because the work runs on the GPU:
 *   - `in`, `out` and `temp` may be host pointers (staged through device memory; pinned host memory from
 *     kfr_allocate copies fastest) or device pointers (used in place).  The call returns when the result
 *     is in `out`, as the reference's does.
 *   - `temp` is device scratch: a device pointer of at least *_get_temp_size bytes is used as scratch; a
 *     NULL or host pointer makes the plan use scratch of its own.
 *
 * The second part declares additive extensions (batched and stream-ordered execution) that have no
 * reference counterpart.
 */
#ifndef KFR_GB300_CAPI_H
#define KFR_GB300_CAPI_H

#include <stddef.h>
#include <stdint.h>

#if defined __STDC_IEC_559_COMPLEX__ && !defined KFR_NO_C_COMPLEX_TYPES
#include <complex.h>
#endif

#ifdef __cplusplus
extern "C"
{
#endif

#if defined(_WIN32)
#define KFR_API_SPEC __declspec(dllexport)
#else
#define KFR_API_SPEC __attribute__((visibility("default")))
#endif

/* kfr_bool as in include/kfr/capi.h:79-95 */
#if defined(__STDC_VERSION__) && __STDC_VERSION__ >= 199901L
typedef _Bool kfr_bool;
#elif defined(__cplusplus)
typedef bool kfr_bool;
#else
typedef char kfr_bool;
#endif

/* scalar and complex element types, include/kfr/capi.h:131-143 */
typedef float kfr_f32;
typedef double kfr_f64;
#if defined __STDC_IEC_559_COMPLEX__ && !defined KFR_NO_C_COMPLEX_TYPES
typedef float _Complex kfr_c32;
typedef double _Complex kfr_c64;
#define KFR_COMPLEX_SIZE_MULTIPLIER 1
#else
typedef float kfr_c32;
typedef double kfr_c64;
#define KFR_COMPLEX_SIZE_MULTIPLIER 2
#endif

/* opaque plan handles, include/kfr/capi.h:145-161 */
#define KFR_OPAQUE_STRUCT(NAME)                                                                             \
    typedef struct NAME                                                                                     \
    {                                                                                                       \
        int opaque;                                                                                         \
    } NAME;
KFR_OPAQUE_STRUCT(KFR_DFT_PLAN_F32)
KFR_OPAQUE_STRUCT(KFR_DFT_PLAN_F64)
KFR_OPAQUE_STRUCT(KFR_DFT_REAL_PLAN_F32)
KFR_OPAQUE_STRUCT(KFR_DFT_REAL_PLAN_F64)
KFR_OPAQUE_STRUCT(KFR_DCT_PLAN_F32)
KFR_OPAQUE_STRUCT(KFR_DCT_PLAN_F64)
KFR_OPAQUE_STRUCT(KFR_FILTER_F32)
KFR_OPAQUE_STRUCT(KFR_FILTER_F64)
KFR_OPAQUE_STRUCT(KFR_FILTER_C32)
KFR_OPAQUE_STRUCT(KFR_FILTER_C64)
KFR_OPAQUE_STRUCT(KFR_DFT_UNEVEN_F32) /* uneven batch plan: extension, no counterpart in the reference */

#define KFR_DEFAULT_ALIGNMENT 64 /* include/kfr/capi.h:165 */
#define KFR_HEADERS_VERSION 70000

/* real DFT packing, include/kfr/capi.h:196-200 (values are part of the ABI) */
typedef enum KFR_DFT_PACK_FORMAT
{
    Perm = 0, /* N/2 complex values; X[N/2].re is stored in out[0].im */
    CCs  = 1  /* N/2 + 1 complex values */
} KFR_DFT_PACK_FORMAT;

/* ---- library information and errors ------------------------------------------------------------ */
KFR_API_SPEC const char* kfr_version_string(void); /* capi.h:116 */
KFR_API_SPEC uint32_t kfr_version(void);           /* capi.h:119: 70001 */
KFR_API_SPEC const char* kfr_enabled_archs(void);  /* capi.h:122: "sm_103a" */
KFR_API_SPEC int kfr_current_arch(void);           /* capi.h:125: compute capability, e.g. 103 */
KFR_API_SPEC const char* kfr_last_error(void);     /* capi.h:128: thread-local, "" after a success */

/* ---- host memory (pinned when a GPU is present, so staging copies run at DMA speed) ----------- */
KFR_API_SPEC void* kfr_allocate(size_t size);                           /* capi.h:170 */
KFR_API_SPEC void* kfr_allocate_aligned(size_t size, size_t alignment); /* capi.h:173 */
KFR_API_SPEC void kfr_deallocate(void* ptr);                            /* capi.h:176 */
/* The reference's managed-allocation helpers (capi.h:178-193, src/capi/capi.cpp:200-216), always exported
 * here.  A block starts with one reference; kfr_deallocate and kfr_release drop one and free the block at
 * zero; kfr_reallocate* copy min(old, new) bytes into a new block and release the old one (new_size 0:
 * release and return NULL; ptr NULL: plain allocation). */
KFR_API_SPEC void* kfr_reallocate(void* ptr, size_t new_size);                             /* capi.h:180 */
KFR_API_SPEC void* kfr_reallocate_aligned(void* ptr, size_t new_size, size_t alignment);   /* capi.h:183 */
KFR_API_SPEC void* kfr_add_ref(void* ptr);                                                 /* capi.h:186 */
KFR_API_SPEC void kfr_release(void* ptr);                                                  /* capi.h:189 */
KFR_API_SPEC size_t kfr_allocated_size(void* ptr);                                         /* capi.h:192 */

/* ---- complex DFT ---------------------------------------------------------------------------------- */
KFR_API_SPEC KFR_DFT_PLAN_F32* kfr_dft_create_plan_f32(size_t size);                              /* capi.h:207 */
KFR_API_SPEC KFR_DFT_PLAN_F32* kfr_dft_create_2d_plan_f32(size_t size1, size_t size2);            /* capi.h:215 */
KFR_API_SPEC KFR_DFT_PLAN_F32* kfr_dft_create_3d_plan_f32(size_t size1, size_t size2, size_t size3); /* capi.h:224 */
KFR_API_SPEC KFR_DFT_PLAN_F32* kfr_dft_create_md_plan_f32(size_t dims, const unsigned* shape);    /* capi.h:232 */
KFR_API_SPEC KFR_DFT_PLAN_F64* kfr_dft_create_plan_f64(size_t size);                              /* capi.h:239 */
KFR_API_SPEC KFR_DFT_PLAN_F64* kfr_dft_create_2d_plan_f64(size_t size1, size_t size2);            /* capi.h:247 */
KFR_API_SPEC KFR_DFT_PLAN_F64* kfr_dft_create_3d_plan_f64(size_t size1, size_t size2, size_t size3); /* capi.h:256 */
KFR_API_SPEC KFR_DFT_PLAN_F64* kfr_dft_create_md_plan_f64(size_t dims, const unsigned* shape);    /* capi.h:264 */
KFR_API_SPEC void kfr_dft_dump_f32(KFR_DFT_PLAN_F32* plan);                                       /* capi.h:270 */
KFR_API_SPEC void kfr_dft_dump_f64(KFR_DFT_PLAN_F64* plan);                                       /* capi.h:276 */
KFR_API_SPEC size_t kfr_dft_get_size_f32(KFR_DFT_PLAN_F32* plan);                                 /* capi.h:283 */
KFR_API_SPEC size_t kfr_dft_get_size_f64(KFR_DFT_PLAN_F64* plan);                                 /* capi.h:290 */
KFR_API_SPEC size_t kfr_dft_get_temp_size_f32(KFR_DFT_PLAN_F32* plan);                            /* capi.h:299 */
KFR_API_SPEC size_t kfr_dft_get_temp_size_f64(KFR_DFT_PLAN_F64* plan);                            /* capi.h:308 */
KFR_API_SPEC void kfr_dft_execute_f32(KFR_DFT_PLAN_F32* plan, kfr_c32* out, const kfr_c32* in,
                                      uint8_t* temp); /* capi.h:320 */
KFR_API_SPEC void kfr_dft_execute_f64(KFR_DFT_PLAN_F64* plan, kfr_c64* out, const kfr_c64* in,
                                      uint8_t* temp); /* capi.h:333 */
KFR_API_SPEC void kfr_dft_execute_inverse_f32(KFR_DFT_PLAN_F32* plan, kfr_c32* out, const kfr_c32* in,
                                              uint8_t* temp); /* capi.h:346 */
KFR_API_SPEC void kfr_dft_execute_inverse_f64(KFR_DFT_PLAN_F64* plan, kfr_c64* out, const kfr_c64* in,
                                              uint8_t* temp); /* capi.h:359 */
KFR_API_SPEC void kfr_dft_delete_plan_f32(KFR_DFT_PLAN_F32* plan); /* capi.h:366 */
KFR_API_SPEC void kfr_dft_delete_plan_f64(KFR_DFT_PLAN_F64* plan); /* capi.h:372 */

/* ---- real DFT -------------------------------------------------------------------------------------- */
KFR_API_SPEC KFR_DFT_REAL_PLAN_F32* kfr_dft_real_create_plan_f32(size_t size,
                                                                 KFR_DFT_PACK_FORMAT pack_format); /* capi.h:380 */
KFR_API_SPEC KFR_DFT_REAL_PLAN_F32* kfr_dft_real_create_2d_plan_f32(size_t size1, size_t size2,
                                                                    kfr_bool real_out_is_enough); /* capi.h:383 */
KFR_API_SPEC KFR_DFT_REAL_PLAN_F32* kfr_dft_real_create_3d_plan_f32(size_t size1, size_t size2, size_t size3,
                                                                    kfr_bool real_out_is_enough); /* capi.h:385 */
KFR_API_SPEC KFR_DFT_REAL_PLAN_F32* kfr_dft_real_create_md_plan_f32(size_t dims, const unsigned* shape,
                                                                    kfr_bool real_out_is_enough); /* capi.h:387 */
KFR_API_SPEC KFR_DFT_REAL_PLAN_F64* kfr_dft_real_create_plan_f64(size_t size,
                                                                 KFR_DFT_PACK_FORMAT pack_format); /* capi.h:396 */
KFR_API_SPEC KFR_DFT_REAL_PLAN_F64* kfr_dft_real_create_2d_plan_f64(size_t size1, size_t size2,
                                                                    kfr_bool real_out_is_enough); /* capi.h:399 */
KFR_API_SPEC KFR_DFT_REAL_PLAN_F64* kfr_dft_real_create_3d_plan_f64(size_t size1, size_t size2, size_t size3,
                                                                    kfr_bool real_out_is_enough); /* capi.h:401 */
KFR_API_SPEC KFR_DFT_REAL_PLAN_F64* kfr_dft_real_create_md_plan_f64(size_t dims, const unsigned* shape,
                                                                    kfr_bool real_out_is_enough); /* capi.h:403 */
KFR_API_SPEC void kfr_dft_real_dump_f32(KFR_DFT_REAL_PLAN_F32* plan);             /* capi.h:410 */
KFR_API_SPEC void kfr_dft_real_dump_f64(KFR_DFT_REAL_PLAN_F64* plan);             /* capi.h:416 */
KFR_API_SPEC size_t kfr_dft_real_get_size_f32(KFR_DFT_REAL_PLAN_F32* plan);       /* capi.h:423 */
KFR_API_SPEC size_t kfr_dft_real_get_size_f64(KFR_DFT_REAL_PLAN_F64* plan);       /* capi.h:430 */
KFR_API_SPEC size_t kfr_dft_real_get_temp_size_f32(KFR_DFT_REAL_PLAN_F32* plan);  /* capi.h:439 */
KFR_API_SPEC size_t kfr_dft_real_get_temp_size_f64(KFR_DFT_REAL_PLAN_F64* plan);  /* capi.h:448 */
KFR_API_SPEC void kfr_dft_real_execute_f32(KFR_DFT_REAL_PLAN_F32* plan, kfr_c32* out, const kfr_f32* in,
                                           uint8_t* temp); /* capi.h:461 */
KFR_API_SPEC void kfr_dft_real_execute_f64(KFR_DFT_REAL_PLAN_F64* plan, kfr_c64* out, const kfr_f64* in,
                                           uint8_t* temp); /* capi.h:475 */
KFR_API_SPEC void kfr_dft_real_execute_inverse_f32(KFR_DFT_REAL_PLAN_F32* plan, kfr_f32* out, const kfr_c32* in,
                                                   uint8_t* temp); /* capi.h:489 */
KFR_API_SPEC void kfr_dft_real_execute_inverse_f64(KFR_DFT_REAL_PLAN_F64* plan, kfr_f64* out, const kfr_c64* in,
                                                   uint8_t* temp); /* capi.h:503 */
KFR_API_SPEC void kfr_dft_real_delete_plan_f32(KFR_DFT_REAL_PLAN_F32* plan); /* capi.h:510 */
KFR_API_SPEC void kfr_dft_real_delete_plan_f64(KFR_DFT_REAL_PLAN_F64* plan); /* capi.h:516 */

/* ---- DCT-II / DCT-III ----------------------------------------------------------------------------- */
KFR_API_SPEC KFR_DCT_PLAN_F32* kfr_dct_create_plan_f32(size_t size);     /* capi.h:523 */
KFR_API_SPEC KFR_DCT_PLAN_F64* kfr_dct_create_plan_f64(size_t size);     /* capi.h:530 */
KFR_API_SPEC void kfr_dct_dump_f32(KFR_DCT_PLAN_F32* plan);              /* capi.h:536 */
KFR_API_SPEC void kfr_dct_dump_f64(KFR_DCT_PLAN_F64* plan);              /* capi.h:542 */
KFR_API_SPEC size_t kfr_dct_get_size_f32(KFR_DCT_PLAN_F32* plan);        /* capi.h:549 */
KFR_API_SPEC size_t kfr_dct_get_size_f64(KFR_DCT_PLAN_F64* plan);        /* capi.h:556 */
KFR_API_SPEC size_t kfr_dct_get_temp_size_f32(KFR_DCT_PLAN_F32* plan);   /* capi.h:565 */
KFR_API_SPEC size_t kfr_dct_get_temp_size_f64(KFR_DCT_PLAN_F64* plan);   /* capi.h:574 */
KFR_API_SPEC void kfr_dct_execute_f32(KFR_DCT_PLAN_F32* plan, kfr_f32* out, const kfr_f32* in,
                                      uint8_t* temp); /* capi.h:586 */
KFR_API_SPEC void kfr_dct_execute_f64(KFR_DCT_PLAN_F64* plan, kfr_f64* out, const kfr_f64* in,
                                      uint8_t* temp); /* capi.h:598 */
KFR_API_SPEC void kfr_dct_execute_inverse_f32(KFR_DCT_PLAN_F32* plan, kfr_f32* out, const kfr_f32* in,
                                              uint8_t* temp); /* capi.h:610 */
KFR_API_SPEC void kfr_dct_execute_inverse_f64(KFR_DCT_PLAN_F64* plan, kfr_f64* out, const kfr_f64* in,
                                              uint8_t* temp); /* capi.h:623 */
KFR_API_SPEC void kfr_dct_delete_plan_f32(KFR_DCT_PLAN_F32* plan); /* capi.h:630 */
KFR_API_SPEC void kfr_dct_delete_plan_f64(KFR_DCT_PLAN_F64* plan); /* capi.h:636 */

/* ---- filters ------------------------------------------------------------------------------------------
 * The FFT convolution filter (convolve_filter) is the GPU path.  FIR plans run through it too: the
 * reference's fir_filter and convolve_filter compute the same y[n] = sum_k taps[k] x[n - k] with state kept
 * across process calls (docs/docs/fir.md:94), so a FIR plan is a convolution filter with the default block;
 * results match the direct form to floating-point rounding.  The IIR creators are declared for link
 * compatibility; IIR filtering is not DFT work, is not built here and returns NULL with an error message. */
KFR_API_SPEC KFR_FILTER_F32* kfr_filter_create_fir_plan_f32(const kfr_f32* taps, size_t size); /* capi.h:644 */
KFR_API_SPEC KFR_FILTER_F64* kfr_filter_create_fir_plan_f64(const kfr_f64* taps, size_t size); /* capi.h:652 */
KFR_API_SPEC KFR_FILTER_F32* kfr_filter_create_convolution_plan_f32(const kfr_f32* taps, size_t size,
                                                                    size_t block_size); /* capi.h:663 */
KFR_API_SPEC KFR_FILTER_F64* kfr_filter_create_convolution_plan_f64(const kfr_f64* taps, size_t size,
                                                                    size_t block_size); /* capi.h:675 */
KFR_API_SPEC KFR_FILTER_F32* kfr_filter_create_iir_plan_f32(const kfr_f32* sos, size_t sos_count); /* capi.h:684 */
KFR_API_SPEC KFR_FILTER_F64* kfr_filter_create_iir_plan_f64(const kfr_f64* sos, size_t sos_count); /* capi.h:692 */
KFR_API_SPEC void kfr_filter_process_f32(KFR_FILTER_F32* plan, kfr_f32* output, const kfr_f32* input,
                                         size_t size); /* capi.h:701 */
KFR_API_SPEC void kfr_filter_process_f64(KFR_FILTER_F64* plan, kfr_f64* output, const kfr_f64* input,
                                         size_t size); /* capi.h:711 */
KFR_API_SPEC void kfr_filter_reset_f32(KFR_FILTER_F32* plan);       /* capi.h:718 */
KFR_API_SPEC void kfr_filter_reset_f64(KFR_FILTER_F64* plan);       /* capi.h:724 */
KFR_API_SPEC void kfr_filter_delete_plan_f32(KFR_FILTER_F32* plan); /* capi.h:730 */
KFR_API_SPEC void kfr_filter_delete_plan_f64(KFR_FILTER_F64* plan); /* capi.h:736 */

/* ======================================================================================================
 * Extensions (no counterpart in the reference).
 *
 * Batched execution runs `batch` independent signals back to back in memory with one launch sequence:
 * signal b of a complex plan starts at in + b*N; of a real plan at in + b*N (reals) and
 * out + b*(N/2+1 or N/2) (complex); of a DCT plan at b*N.  `stream`: NULL runs synchronously (host or
 * device pointers, like the single-signal calls); otherwise it is a cudaStream_t and the call only enqueues
 * work on it, so all three pointers must be device memory and the caller synchronises.  temp: NULL or host
 * uses plan-owned scratch (then calls on one plan must not overlap in time); a device pointer of
 * *_get_temp_size_batch bytes is used instead.
 * ====================================================================================================== */
KFR_API_SPEC size_t kfr_dft_get_temp_size_batch_f32(KFR_DFT_PLAN_F32* plan, size_t batch);
KFR_API_SPEC size_t kfr_dft_get_temp_size_batch_f64(KFR_DFT_PLAN_F64* plan, size_t batch);
KFR_API_SPEC void kfr_dft_execute_batch_f32(KFR_DFT_PLAN_F32* plan, size_t batch, kfr_c32* out, const kfr_c32* in,
                                            uint8_t* temp, kfr_bool inverse, void* stream);
KFR_API_SPEC void kfr_dft_execute_batch_f64(KFR_DFT_PLAN_F64* plan, size_t batch, kfr_c64* out, const kfr_c64* in,
                                            uint8_t* temp, kfr_bool inverse, void* stream);

KFR_API_SPEC size_t kfr_dft_real_get_temp_size_batch_f32(KFR_DFT_REAL_PLAN_F32* plan, size_t batch);
KFR_API_SPEC size_t kfr_dft_real_get_temp_size_batch_f64(KFR_DFT_REAL_PLAN_F64* plan, size_t batch);
KFR_API_SPEC void kfr_dft_real_execute_batch_f32(KFR_DFT_REAL_PLAN_F32* plan, size_t batch, kfr_c32* out,
                                                 const kfr_f32* in, uint8_t* temp, void* stream);
KFR_API_SPEC void kfr_dft_real_execute_batch_f64(KFR_DFT_REAL_PLAN_F64* plan, size_t batch, kfr_c64* out,
                                                 const kfr_f64* in, uint8_t* temp, void* stream);
KFR_API_SPEC void kfr_dft_real_execute_inverse_batch_f32(KFR_DFT_REAL_PLAN_F32* plan, size_t batch, kfr_f32* out,
                                                         const kfr_c32* in, uint8_t* temp, void* stream);
KFR_API_SPEC void kfr_dft_real_execute_inverse_batch_f64(KFR_DFT_REAL_PLAN_F64* plan, size_t batch, kfr_f64* out,
                                                         const kfr_c64* in, uint8_t* temp, void* stream);

KFR_API_SPEC size_t kfr_dct_get_temp_size_batch_f32(KFR_DCT_PLAN_F32* plan, size_t batch);
KFR_API_SPEC size_t kfr_dct_get_temp_size_batch_f64(KFR_DCT_PLAN_F64* plan, size_t batch);
KFR_API_SPEC void kfr_dct_execute_batch_f32(KFR_DCT_PLAN_F32* plan, size_t batch, kfr_f32* out, const kfr_f32* in,
                                            uint8_t* temp, kfr_bool inverse, void* stream);
KFR_API_SPEC void kfr_dct_execute_batch_f64(KFR_DCT_PLAN_F64* plan, size_t batch, kfr_f64* out, const kfr_f64* in,
                                            uint8_t* temp, kfr_bool inverse, void* stream);

/* Whole-signal convolution, correlation and autocorrelation: the reference's C++ convolve / correlate /
 * autocorrelate (include/kfr/dft/convolution.hpp:53-76) as C entry points.  out receives na + nb - 1 values
 * (autocorrelate: n values, lags 0 .. n-1); the return value is that count.  The result is the reference's:
 * the linear convolution computed through DFTs of size next_pow2(na + nb - 1) and scaled by 1/size; for
 * complex inputs only the real part is kept (the imaginary parts of out are zero), as the reference does
 * (src/dft/convolution-impl.cpp:127).  correlate reverses b without conjugating it.  Pointers may be host
 * or device memory; the call is synchronous. */
KFR_API_SPEC size_t kfr_convolve_f32(kfr_f32* out, const kfr_f32* a, size_t na, const kfr_f32* b, size_t nb);
KFR_API_SPEC size_t kfr_convolve_f64(kfr_f64* out, const kfr_f64* a, size_t na, const kfr_f64* b, size_t nb);
KFR_API_SPEC size_t kfr_convolve_c32(kfr_c32* out, const kfr_c32* a, size_t na, const kfr_c32* b, size_t nb);
KFR_API_SPEC size_t kfr_convolve_c64(kfr_c64* out, const kfr_c64* a, size_t na, const kfr_c64* b, size_t nb);
KFR_API_SPEC size_t kfr_correlate_f32(kfr_f32* out, const kfr_f32* a, size_t na, const kfr_f32* b, size_t nb);
KFR_API_SPEC size_t kfr_correlate_f64(kfr_f64* out, const kfr_f64* a, size_t na, const kfr_f64* b, size_t nb);
KFR_API_SPEC size_t kfr_correlate_c32(kfr_c32* out, const kfr_c32* a, size_t na, const kfr_c32* b, size_t nb);
KFR_API_SPEC size_t kfr_correlate_c64(kfr_c64* out, const kfr_c64* a, size_t na, const kfr_c64* b, size_t nb);
KFR_API_SPEC size_t kfr_autocorrelate_f32(kfr_f32* out, const kfr_f32* a, size_t n);
KFR_API_SPEC size_t kfr_autocorrelate_f64(kfr_f64* out, const kfr_f64* a, size_t n);

/* The plan cache behind the convolution entry points (dft_cache, include/kfr/dft/cache.hpp:45-171): number
 * of cached plans, and release of all of them. */
KFR_API_SPEC size_t kfr_dft_cache_size(void);
KFR_API_SPEC void kfr_dft_cache_clear(void);

/* Text description of the plan's GPU strategy (kernel kind, radices, launch shape), as kfr_dft_dump_f32 prints
 * it; copies at most size-1 bytes plus a terminating zero and returns the full length. */
KFR_API_SPEC size_t kfr_dft_describe_f32(KFR_DFT_PLAN_F32* plan, char* buf, size_t size);
KFR_API_SPEC size_t kfr_dft_describe_f64(KFR_DFT_PLAN_F64* plan, char* buf, size_t size);

/* fft_multiply / fft_multiply_accumulate (include/kfr/dft/fft.hpp:983-1020) on device buffers, over `batch`
 * spectra of `size` complex elements stored back to back (the outputs of a real or complex DFT plan):
 *   kfr_fft_multiply_*:            dest = src1 * src2
 *   kfr_fft_multiply_accumulate_*: dest = acc + src1 * src2  (acc == dest is the reference's two-operand
 *                                  form; a separate acc is its three-operand form)
 * fmt = Perm multiplies element 0 part by part (DC and Nyquist, both real, share it), as the reference does.
 * src2_shared != 0: src2 is one spectrum applied to every signal (a filter); else `batch` spectra.  Every
 * pointer must be device memory; dest may alias any input.  stream: NULL = synchronous, else enqueued on
 * that cudaStream_t. */
KFR_API_SPEC void kfr_fft_multiply_f32(kfr_c32* dest, const kfr_c32* src1, const kfr_c32* src2, size_t size,
                                       size_t batch, kfr_bool src2_shared, KFR_DFT_PACK_FORMAT fmt, void* stream);
KFR_API_SPEC void kfr_fft_multiply_f64(kfr_c64* dest, const kfr_c64* src1, const kfr_c64* src2, size_t size,
                                       size_t batch, kfr_bool src2_shared, KFR_DFT_PACK_FORMAT fmt, void* stream);
KFR_API_SPEC void kfr_fft_multiply_accumulate_f32(kfr_c32* dest, const kfr_c32* acc, const kfr_c32* src1,
                                                  const kfr_c32* src2, size_t size, size_t batch,
                                                  kfr_bool src2_shared, KFR_DFT_PACK_FORMAT fmt, void* stream);
KFR_API_SPEC void kfr_fft_multiply_accumulate_f64(kfr_c64* dest, const kfr_c64* acc, const kfr_c64* src1,
                                                  const kfr_c64* src2, size_t size, size_t batch,
                                                  kfr_bool src2_shared, KFR_DFT_PACK_FORMAT fmt, void* stream);

/* Progressive execution (dft_plan<T>::progressive_*, include/kfr/dft/fft.hpp:393-439): the reference runs
 * one stage per step; here one step is one kernel launch of the plan, run to completion.
 *   total_steps: the steps of one execution with device buffers aligned as cudaMalloc aligns them;
 *   start:       records the plan's launches for these buffers (nothing runs yet; host buffers are staged:
 *                the input is copied now, the result after the last step) and returns the number of steps
 *                of this execution (it can differ from total_steps for misaligned device pointers);
 *   step:        runs step `step` (0, 1, ... in order) and waits for it; returns nonzero while steps remain.
 *                `out` holds the result after the last step.
 * One progressive execution per plan at a time. */
KFR_API_SPEC size_t kfr_dft_progressive_total_steps_f32(KFR_DFT_PLAN_F32* plan);
KFR_API_SPEC size_t kfr_dft_progressive_total_steps_f64(KFR_DFT_PLAN_F64* plan);
KFR_API_SPEC size_t kfr_dft_progressive_start_f32(KFR_DFT_PLAN_F32* plan, kfr_c32* out, const kfr_c32* in,
                                                  uint8_t* temp, kfr_bool inverse);
KFR_API_SPEC size_t kfr_dft_progressive_start_f64(KFR_DFT_PLAN_F64* plan, kfr_c64* out, const kfr_c64* in,
                                                  uint8_t* temp, kfr_bool inverse);
KFR_API_SPEC kfr_bool kfr_dft_progressive_step_f32(KFR_DFT_PLAN_F32* plan, size_t step);
KFR_API_SPEC kfr_bool kfr_dft_progressive_step_f64(KFR_DFT_PLAN_F64* plan, size_t step);

/* Number of kernel launches one batched execute of this plan issues (forward direction). */
KFR_API_SPEC size_t kfr_dft_get_launch_count_f32(KFR_DFT_PLAN_F32* plan, size_t batch);
KFR_API_SPEC size_t kfr_dft_get_launch_count_f64(KFR_DFT_PLAN_F64* plan, size_t batch);

/* Multi-channel convolution filter (no counterpart in the reference, whose filters are single-channel): the
 * same filter applied independently to `channels` signals, each with its own state.  kfr_filter_process_*
 * on such a plan takes channels * size samples, channel-major (channel c at c * size), and runs every block of
 * every channel in one launch; kfr_filter_reset_* clears every channel's state. */
KFR_API_SPEC KFR_FILTER_F32* kfr_filter_create_convolution_plan_channels_f32(const kfr_f32* taps, size_t size,
                                                                           size_t block_size, size_t channels);
KFR_API_SPEC KFR_FILTER_F64* kfr_filter_create_convolution_plan_channels_f64(const kfr_f64* taps, size_t size,
                                                                           size_t block_size, size_t channels);

/* Tensor-core plans (no counterpart in the reference): a complex plan whose radix-16 passes run on the tensor
 * cores as DFT-matrix contractions with each FP32 operand split into 16-bit parts, products accumulated in
 * FP32.  split = 1: three BF16 parts (hi + mid + lo), the six products down to 2^-16 of the leading one;
 * split = 2: FP16 hi + lo after a power-of-two scaling of each butterfly's inputs, products hi*hi + hi*lo +
 * lo*hi.  Lengths 256 and 4096 (one CTA per signal group) and 65536 = 256 x 256, 2^20 = 256 x 4096 and
 * 2^24 = 4096 x 4096 (four-step: scratch of one signal per signal, like the CUDA-core four-step).  The handle
 * is an ordinary KFR_DFT_PLAN_F32 (execute, batch, describe, delete as usual); the tests report its error
 * against FP64 beside the FP32 CUDA-core plan's. */
KFR_API_SPEC KFR_DFT_PLAN_F32* kfr_dft_create_plan_tensor_f32(size_t size, int split);

/* Uneven batch (no counterpart in the reference, whose callers loop over one plan per length): `count` complex
 * signals of the given lengths stored back to back, transformed by one persistent work-queue launch (plus
 * regular launches for signals too long for one CTA), replayed as a CUDA graph after the first call with a
 * given (out, in, direction).  autotune: time candidate radix orders and tiles per length class when the
 * plan is created (the choice is cached for the process).  in and out are device pointers (count * total
 * elements, see kfr_dft_uneven_get_size_f32); stream: NULL = default stream, synchronous.
 * kfr_dft_uneven_execute_per_signal_f32 runs the same transforms as one regular plan execution per signal
 * (the plain form, for comparison). */
KFR_API_SPEC KFR_DFT_UNEVEN_F32* kfr_dft_create_uneven_plan_f32(const size_t* lengths, size_t count, kfr_bool autotune);
KFR_API_SPEC size_t kfr_dft_uneven_get_size_f32(KFR_DFT_UNEVEN_F32* plan);
KFR_API_SPEC void kfr_dft_uneven_execute_f32(KFR_DFT_UNEVEN_F32* plan, kfr_c32* out, const kfr_c32* in, kfr_bool inverse,
                                             void* stream);
KFR_API_SPEC void kfr_dft_uneven_execute_per_signal_f32(KFR_DFT_UNEVEN_F32* plan, kfr_c32* out, const kfr_c32* in,
                                                        kfr_bool inverse, void* stream);
KFR_API_SPEC size_t kfr_dft_uneven_describe_f32(KFR_DFT_UNEVEN_F32* plan, char* buf, size_t size);
KFR_API_SPEC void kfr_dft_uneven_delete_plan_f32(KFR_DFT_UNEVEN_F32* plan);

/* Failure detection (no counterpart in the reference).  Every wait of a kernel -- for a bulk copy into its
 * shared memory, or (uneven batch) for an earlier stage of its signal -- gives up after a bounded number of
 * polling rounds.  The kernel then sets its plan's device error flag, lets its own copies in flight land
 * (waiting at most the default limit again) and returns or carries on; the next synchronous call on that plan
 * reports "... gave up waiting ..." through kfr_last_error() and clears the flag.  With a stream, the flag is
 * read by the next synchronous call on the same plan.
 *   kfr_set_wait_limit: polling rounds for launches issued from now on (KFR_DEFAULT_WAIT_SPINS, about a
 *     second or more; 0 makes every wait give up at its first poll, for tests); returns the previous value.
 *   kfr_dft_uneven_set_unreachable_stage_f32: test hook; nonzero makes every tile that depends on an earlier
 *     stage wait for one more tile than that stage has, so the wait runs out after the limit. */
#define KFR_DEFAULT_WAIT_SPINS (1u << 22)
KFR_API_SPEC uint32_t kfr_set_wait_limit(uint32_t spins);
KFR_API_SPEC void kfr_dft_uneven_set_unreachable_stage_f32(KFR_DFT_UNEVEN_F32* plan, kfr_bool unreachable);

/* Adjoints (vector-Jacobian products) for gradient-based callers; no counterpart in the reference, which has
 * no differentiation.  Each maps the gradient of a transform's output (grad_out) to the gradient of its input
 * (grad_in), batch signals laid out as in the batched calls above, with the same pointer and stream rules
 * (the real and DCT adjoints keep their scratch in the plan and ignore temp).  Complex gradients follow the complex-autograd convention: for a real loss L the gradient of a
 * complex value z is dL/dRe(z) + i dL/dIm(z).
 *   kfr_dft_adjoint_batch:              of execute (inverse = 0) or execute_inverse (inverse = 1): the
 *                                       unscaled transform in the other direction;
 *   kfr_dft_real_adjoint_batch:         of the forward real DFT: the inverse real DFT of grad_out with bins
 *                                       1 .. N/2-1 halved (one-dimensional plans);
 *   kfr_dft_real_adjoint_inverse_batch: of the inverse real DFT: the forward real DFT of grad_out with bins
 *                                       1 .. N/2-1 doubled (one-dimensional plans);
 *   kfr_dct_adjoint_batch:              of the DCT-II (inverse = 0: DCT-III of grad_out with its first value
 *                                       doubled) or of the reference's DCT-III (inverse = 1: DCT-II, then the
 *                                       first value halved). */
KFR_API_SPEC void kfr_dft_adjoint_batch_f32(KFR_DFT_PLAN_F32* plan, size_t batch, kfr_c32* grad_in,
                                            const kfr_c32* grad_out, uint8_t* temp, kfr_bool inverse, void* stream);
KFR_API_SPEC void kfr_dft_adjoint_batch_f64(KFR_DFT_PLAN_F64* plan, size_t batch, kfr_c64* grad_in,
                                            const kfr_c64* grad_out, uint8_t* temp, kfr_bool inverse, void* stream);
KFR_API_SPEC void kfr_dft_real_adjoint_batch_f32(KFR_DFT_REAL_PLAN_F32* plan, size_t batch, kfr_f32* grad_in,
                                                 const kfr_c32* grad_out, uint8_t* temp, void* stream);
KFR_API_SPEC void kfr_dft_real_adjoint_batch_f64(KFR_DFT_REAL_PLAN_F64* plan, size_t batch, kfr_f64* grad_in,
                                                 const kfr_c64* grad_out, uint8_t* temp, void* stream);
KFR_API_SPEC void kfr_dft_real_adjoint_inverse_batch_f32(KFR_DFT_REAL_PLAN_F32* plan, size_t batch, kfr_c32* grad_in,
                                                         const kfr_f32* grad_out, uint8_t* temp, void* stream);
KFR_API_SPEC void kfr_dft_real_adjoint_inverse_batch_f64(KFR_DFT_REAL_PLAN_F64* plan, size_t batch, kfr_c64* grad_in,
                                                         const kfr_f64* grad_out, uint8_t* temp, void* stream);
KFR_API_SPEC void kfr_dct_adjoint_batch_f32(KFR_DCT_PLAN_F32* plan, size_t batch, kfr_f32* grad_in,
                                            const kfr_f32* grad_out, uint8_t* temp, kfr_bool inverse, void* stream);
KFR_API_SPEC void kfr_dct_adjoint_batch_f64(KFR_DCT_PLAN_F64* plan, size_t batch, kfr_f64* grad_in,
                                            const kfr_f64* grad_out, uint8_t* temp, kfr_bool inverse, void* stream);

/* Gradients of the causal FIR convolution that a convolution filter (kfr_filter_create_convolution_plan) applies
 * from a reset state, y[c][t] = sum_{m<ntaps} taps[m] x[c][t-m], over `channels` signals of n samples each
 * (channel-major): grad_x[c][t] = sum_m taps[m] grad_y[c][t+m] and grad_taps[m] = sum_c sum_t grad_y[c][t]
 * x[c][t-m].  Device pointers only; grad_x or grad_taps may be NULL when not wanted.  stream: NULL = default
 * stream; the call returns when the gradients are written. */
KFR_API_SPEC void kfr_fir_backward_f32(const kfr_f32* taps, size_t ntaps, size_t channels, size_t n, const kfr_f32* x,
                                       const kfr_f32* grad_y, kfr_f32* grad_x, kfr_f32* grad_taps, void* stream);
KFR_API_SPEC void kfr_fir_backward_f64(const kfr_f64* taps, size_t ntaps, size_t channels, size_t n, const kfr_f64* x,
                                       const kfr_f64* grad_y, kfr_f64* grad_x, kfr_f64* grad_taps, void* stream);

/* Allocation-free execution (no counterpart in the reference).
 *
 * Same transform as kfr_dft_execute_batch_f32, for callers that must not allocate GPU memory while they
 * run: real-time audio or control threads, code inside CUDA stream capture, and hosts that reserve all
 * device memory up front.  kfr_dft_execute_batch_f32 allocates plan-owned scratch on first use (and
 * staging buffers for host pointers); this entry point never calls cudaMalloc, cudaFree or any other
 * allocating routine.  Plans whose length needs scratch (the two-pass path for long transforms and the
 * multi-kernel Bluestein path) use one fixed device array of KFR_STATIC_SCRATCH_BYTES that the library
 * holds on every GPU it runs on until the process exits.
 *   - in and out must be device pointers (host pointers would need staging buffers): error otherwise;
 *   - batch * the plan's per-signal scratch must fit KFR_STATIC_SCRATCH_BYTES: error otherwise
 *     (kfr_dft_get_temp_size_batch_f32 gives the requirement);
 *   - stream: NULL = synchronous on the default stream, else a cudaStream_t the work is enqueued on;
 *   - the first call on each device, whatever the plan, does the one-time set-up (looks up the array's
 *     device address): make that first call before any stream capture;
 *   - the CUDA driver loads each kernel's code on its first launch, and that load takes device memory: run
 *     each plan once through this entry point, with the batch it will use, before stream capture or
 *     real-time use;
 *   - every call shares the one array and no call needs it cleared; calls that overlap on the GPU (on
 *     different streams, or from different threads) race on it and must be serialised by the caller.
 * Errors are reported through kfr_last_error() like every other entry point. */
#define KFR_STATIC_SCRATCH_BYTES (32u << 20)
KFR_API_SPEC void kfr_dft_execute_static_scratch_f32(KFR_DFT_PLAN_F32* plan, size_t batch, kfr_c32* out,
                                                     const kfr_c32* in, kfr_bool inverse, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* KFR_GB300_CAPI_H */
