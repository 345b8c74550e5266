/*
 * p3dfft_gb300.h -- explicit device API of the GB300 P3DFFT transform library.
 *
 * Plain C ABI (no CUDA or torch types in the signatures).  Arrays passed to
 * the transform calls are DEVICE pointers; the stream argument is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).  Every
 * call returns 0 on success or a negative P3G_E* code; p3g_last_error()
 * returns the message of the last failure on the calling thread.
 *
 * The drop-in reference interface (p3dfft_setup, p3dfft_ftran_r2c, ...) is
 * declared in p3dfft.h and implemented on top of this API by libp3dfft.so.
 *
 * Array layouts follow the reference (column-major, X fastest):
 *   real field     (nx, ny, nz)
 *   complex field  (nxc/2+1, nyc, nzc), interleaved (re, im), or
 *                  (nzc, nyc, nxc/2+1) with P3G_LAYOUT_STRIDE1.
 */
#ifndef P3DFFT_GB300_H
#define P3DFFT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct p3g_plan_s* p3g_plan;

enum {
  P3G_OK = 0,
  P3G_E_ARG = -1,       /* invalid argument (sizes, op letters, geometry) */
  P3G_E_CUDA = -2,      /* a CUDA runtime call failed */
  P3G_E_NOMEM = -3,     /* device allocation failed */
  P3G_E_UNSUPPORTED = -4, /* a size or option outside this build's limits */
  P3G_E_STATE = -5,     /* call out of order (no plan / plan already set up) */
  P3G_E_RANGE = -6      /* F64 path: input magnitudes outside the exponent window at the plan's bias */
};

enum { P3G_F64 = 0, P3G_F32 = 1 };               /* precision of data and arithmetic path */
enum { P3G_LAYOUT_XYZ = 0, P3G_LAYOUT_STRIDE1 = 1 }; /* complex output layout */
enum { P3G_FLAG_TIMERS = 1 };                     /* record per-pass CUDA-event timers */

/* Create a plan for an nx*ny*nz real grid keeping nxc*nyc*nzc modes
 * (pruned transform when smaller than the grid).  Replaces the planning and
 * buffer set-up of p3dfft_setup (reference build/setup.F90:107-605,
 * build/init_plan.F90:29-489): twiddle tables are generated once in FP64 on
 * the host and kept on the device with the stage plans.  The workspace is
 * allocated on the first transform call and grown for larger nv. */
int p3g_plan_create(p3g_plan* plan, int nx, int ny, int nz, int nxc, int nyc, int nzc, int precision, int layout,
                    int flags);
/* p3g_plan_create with the tuning knobs the batch autotuner searches (no
 * counterpart in the reference, whose FFTW planner makes these choices):
 * max_radix caps the power-of-two radix of the FFT stages (2, 4, 8, or 16 on
 * the F32 path; 0 = 8 on F64, 16 on F32) and max_lines caps the lines per
 * shared-memory tile (a power of two; 0 = no cap). */
int p3g_plan_create_tuned(p3g_plan* plan, int nx, int ny, int nz, int nxc, int nyc, int nzc, int precision,
                          int layout, int flags, int max_radix, int max_lines);
int p3g_plan_destroy(p3g_plan plan);

/* Bounds of the local arrays, as p3dfft_get_dims (reference
 * build/module.F90:225-273): conf 1 real space, 2 wavenumber space,
 * 3 padded in-place size (memsize).  1-based start/end, size. */
int p3g_get_dims(p3g_plan plan, int conf, int start[3], int end[3], int size[3]);

/* Forward real-to-complex transform of nv fields (reference
 * build/ftran.F90:489-780 and :104-317).  op is 3 letters; op[2] selects the
 * Z transform: 't'/'f' FFT, 'c' DCT-I (REDFT00), 's' DST-I (RODFT00), 'n'/'0'
 * none.  dim_in/dim_out are the element spacings between fields (reals /
 * complexes); <= 0 selects the dense size.  in and out may alias. */
int p3g_ftran_r2c(p3g_plan plan, const void* in, void* out, const char* op, int nv, long long dim_in,
                  long long dim_out, void* stream);

/* Backward complex-to-real transform (reference build/btran.F90:396-679 and
 * :104-304); op[0] selects the Z transform.  Unnormalised.  The input is not
 * modified. */
int p3g_btran_c2r(p3g_plan plan, const void* in, void* out, const char* op, int nv, long long dim_in,
                  long long dim_out, void* stream);

/* Single-field transforms between a device (or GPU-addressable host) real
 * array and a HOST complex array, with the host copies overlapped with the Z
 * pass (no counterpart in the reference, whose arrays are host memory
 * throughout): ftran runs X and Y, then the Z pass in `chunks` row blocks,
 * copying each block's output to out_host on copy_stream while the next block
 * computes; btran copies the input in row blocks and starts each block's Z pass
 * when its copy has landed.  stage is a device buffer of the complex array's
 * size.  XYZ layout.  The caller synchronises both streams. */
int p3g_ftran_r2c_to_host(p3g_plan plan, const void* in, void* out_host, void* stage, const char* op, int chunks,
                          void* stream, void* copy_stream);
int p3g_btran_c2r_from_host(p3g_plan plan, const void* in_host, void* stage, void* out, const char* op, int chunks,
                            void* stream, void* copy_stream);

/* p3dfft_ftran_r2c_1d (reference build/ftran.F90:787-814): the real-to-
 * complex X transform alone, every (y, z) line of the real field in to
 * nx/2+1 complexes per line out, lines packed (complex (nx/2+1, ny, nz),
 * user format), unnormalised and not pruned. */
int p3g_ftran_r2c_1d(p3g_plan plan, const void* in, void* out, void* stream);

/* p3dfft_cheby (reference build/ftran.F90:321-464): 'ffc' transform, scaling
 * by 1/(nx*ny*(nzc-1)) and the Chebyshev-derivative recurrence along z with
 * factor 4/lz. */
int p3g_cheby(p3g_plan plan, const void* in, void* out, double lz, int nv, long long dim_in, long long dim_out,
              void* stream);

/* Shell spectrum of a forward transform's output `in` (device, ip=2 layout),
 * restating compute_spectrum of the reference's spectrum sample
 * (sample/FORTRAN/driver_spec.F90:263-341) for one rank.  For each of nv
 * fields, E[f*(kmax+1) + ik] (device, binary64) = scale^2 * sum of
 * weight * |B|^2 over the kept modes with ik = int(sqrt(kx^2+ky^2+kz^2)+0.5),
 * ky and kz folded to |frequency| as the sample folds them.  weight is k^2
 * with P3G_SPEC_K2 (the sample's choice), else 1, and is doubled with
 * P3G_SPEC_HERMITIAN for modes 0 < kx, 2 kx != nx (the conjugate half of a
 * real field).  Accumulated in binary64; E is cleared first.  kmax <= 0
 * selects the sample's int(sqrt(nx^2+ny^2+nz^2)/2 + 0.5); a kmax below the
 * sample's own check (driver_spec.F90:271-274) is an error, and modes beyond
 * kmax are not counted. */
enum { P3G_SPEC_K2 = 1, P3G_SPEC_HERMITIAN = 2 };
int p3g_spectrum(p3g_plan plan, const void* in, double* E, int kmax, double scale, int flags, int nv,
                 long long dim_in, void* stream);

/* ---------------------------------------------------------------------
 * Batches: many independent transforms of different sizes in one persistent
 * launch (no counterpart in the reference, which transforms one grid per
 * call).  Each job runs on its own plan (XYZ or STRIDE1 layout, pruning
 * allowed, Z transform 'fft') with its own device work buffer of
 * p3g_job_work_bytes(plan, kind) bytes:
 *   P3G_JOB_ROUNDTRIP  in real -> forward -> (complex kept in work) ->
 *                      backward -> out real (unnormalised, as the reference)
 *   P3G_JOB_FORWARD    in real -> out complex
 *   P3G_JOB_BACKWARD   in complex -> out real (in is not modified)
 *   P3G_JOB_SPECTRUM   in real -> forward (complex kept in work) ->
 *                      out double[kmax+1] shell spectrum (p3g_spectrum with
 *                      kmax, scale, flags)
 * p3g_batch_set_jobs builds the work queue (jobs in windows of `window`,
 * pass-major inside a window; <= 0 = one window) in page-locked staging,
 * without waiting for the device; p3g_batch_launch enqueues on a stream the
 * queue's upload (after the previous launch of the batch, on whichever
 * stream), the launch and the copy of its status words; p3g_batch_capture
 * uploads the queue and records the launch as a CUDA graph that
 * p3g_batch_replay launches.  The job arrays are bound at set_jobs time;
 * the caller keeps them alive and unchanged until the launches that use them
 * have finished.  One precision per batch. */
enum { P3G_JOB_ROUNDTRIP = 0, P3G_JOB_FORWARD = 1, P3G_JOB_BACKWARD = 2, P3G_JOB_SPECTRUM = 3 };
typedef struct {
  p3g_plan plan;
  int kind;
  int kmax;      /* spectrum: bins - 1 (<= 0 selects the sample's default) */
  int flags;     /* spectrum: P3G_SPEC_* */
  int reserved;
  double scale;  /* spectrum: B is multiplied by scale before squaring */
  const void* in;
  void* out;
  void* work;
} p3g_job;
typedef struct p3g_batch_s* p3g_batch;
long long p3g_job_work_bytes(p3g_plan plan, int kind);
int p3g_batch_create(p3g_batch* batch, int precision);
int p3g_batch_set_jobs(p3g_batch batch, int njobs, const p3g_job* jobs, int window);
int p3g_batch_launch(p3g_batch batch, void* stream);
int p3g_batch_capture(p3g_batch batch);
int p3g_batch_replay(p3g_batch batch, void* stream);
/* Synchronises the stream and the batch's last launch, then reports a
 * timed-out dependency wait, or P3G_E_RANGE for F64 jobs whose binary64
 * inputs left their plans' exponent window. */
int p3g_batch_status(p3g_batch batch, void* stream);
/* info = {passes, work items, persistent CTAs, launches so far, threads per
 * CTA (128, or 256 when a line is longer than 2048 points)} */
int p3g_batch_info(p3g_batch batch, long long info[5]);
/* Test hook for the bounded dependency waits: makes the passes that depend
 * on pass `pass` (queue order, as numbered by set_jobs) wait for a tile that
 * never completes, so their waits run out (about 4 s) and the next
 * p3g_batch_status reports the time-out; the launch ends and the context stays
 * usable.  The next p3g_batch_set_jobs clears it. */
int p3g_batch_block_pass(p3g_batch batch, int pass);
int p3g_batch_destroy(p3g_batch batch);

/* The reference's 12 accumulating stage timers (build/module.F90:106,709-744),
 * in seconds: slot 5 X r2c, 7 Y forward, 8 Z forward, 9 Z backward,
 * 10 Y backward, 12 X c2r (1-based; communication slots stay 0).  Needs
 * P3G_FLAG_TIMERS; get synchronises with the recorded events. */
int p3g_get_timers(p3g_plan plan, double timers[12]);
int p3g_set_timers(p3g_plan plan);

/* Device bytes held by the plan (tables + workspace). */
long long p3g_plan_device_bytes(p3g_plan plan);
/* Kernel launches issued by this plan since creation. */
long long p3g_plan_launches(p3g_plan plan);

/* Allocation-free forward transform (one field, XYZ or STRIDE1 layout,
 * single-tile kernels).  No counterpart in the reference.  For callers that must not
 * allocate device memory after start-up (fixed-budget serving workers,
 * frameworks that route every allocation through their own pool, loops that
 * cannot afford cudaMalloc's device synchronisation): the workspace is a
 * fixed 32 MiB device array inside the library, not a cudaMalloc.  Grids
 * whose workspace (nz*ny*pitch*16 bytes for F64, *8 for F32, pitch =
 * nxc/2+1 rounded up to 8 resp. 16, plus nz*nyc*pitch*16 resp. 8 when
 * nyc < ny) exceeds it are rejected with P3G_E_UNSUPPORTED.  The plan must exist
 * already (p3g_plan_create allocates).  The first call on each device looks
 * up the array's device address, so make it before any stream capture.
 * All calls share the array: calls that overlap on the GPU race. */
int p3g_ftran_r2c_noalloc(p3g_plan plan, const void* in, void* out, const char* op, void* stream);

/* Binary64 range of the F64 path (no counterpart in the reference, whose
 * FFTW arithmetic is binary64 throughout).  The F64 path computes in
 * double-float, whose exponent range is binary32's, so every F64 transform
 * scales its binary64 input by an exact power of two 2^-k and its output by
 * 2^k.  Results equal the unscaled transform's as long as the largest input
 * magnitude, scaled, lies in [2^-50, 2^(124 - ceil(log2(nx ny 2 (nz+1))))]
 * (the window): k = 0 covers fields of largest magnitude ~1e-15 .. ~1e28 at
 * 1024^3.  Error bounds are relative to the field's largest magnitude;
 * values below 2^-126 of it flush to zero, as they would in any normwise
 * accurate FFT.
 *   P3G_RANGE_FIXED (default): k = bias for every call; the input passes
 *     record the largest magnitude they convert, and p3g_plan_status /
 *     p3g_plan_check_range report P3G_E_RANGE when it was outside the window
 *     (the results of those calls are then invalid; no inf or zero is returned
 *     silently).
 *   P3G_RANGE_AUTO: each call first measures the largest magnitude of its
 *     input on the device (one extra read of the input) and its passes pick k
 *     from it, without a host round trip.
 * The F32 path has binary32's range, as the reference's single-precision
 * build, and ignores these settings. */
enum { P3G_RANGE_FIXED = 0, P3G_RANGE_AUTO = 1 };
int p3g_plan_set_range(p3g_plan plan, int mode, int bias);
/* Synchronises; checks the binary64 inputs converted since the last check
 * against the window at the plan's bias and clears the record.  Returns
 * P3G_OK or P3G_E_RANGE; *bias (may be NULL) receives the bias that brings
 * them into the window (0 when none is needed) and *emax (may be NULL) the
 * largest binary64 exponent seen (-1075 when every input was zero). */
int p3g_plan_check_range(p3g_plan plan, int* bias, int* emax);

/* Synchronises and reports a kernel-side failure recorded on the plan's
 * device flag (a pipelined pass whose bounded wait for a tile copy expired;
 * reported once, then cleared), or P3G_E_RANGE as p3g_plan_check_range
 * (whose record it clears). */
int p3g_plan_status(p3g_plan plan);
/* Test hook for the bounded tile waits (no counterpart in the reference):
 * with on != 0 the pipelined passes' TMA tile barriers expect 16 bytes more
 * than their copies deliver, so every wait runs out (about half a second),
 * the pass records the time-out and ends early, and the next p3g_plan_status
 * reports it (then clears it); on = 0 restores.  Nothing faults and the
 * context stays usable. */
int p3g_plan_block_tiles(p3g_plan plan, int on);
/* Kernel selection: use_pipe = persistent double-buffered passes (default 1),
 * use_tma = TMA tensor-tile copies where the layout allows (default 1).  With
 * both 0 every pass runs the single-tile kernels. */
int p3g_plan_set_options(p3g_plan plan, int use_pipe, int use_tma);

const char* p3g_last_error(void);
int p3g_version(void);

#ifdef __cplusplus
}
#endif
#endif /* P3DFFT_GB300_H */
