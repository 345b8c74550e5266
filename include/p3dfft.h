/*
 * p3dfft.h -- drop-in C interface of the GB300 P3DFFT library (libp3dfft.so,
 * or libp3dfft_single.so when compiled with -DSINGLE_PREC).
 *
 * Same symbols, argument conventions and column-major layouts as the
 * reference header (include/p3dfft.h:120-264 of P3DFFT 2.7): the
 * FORT_MOD_NAME(...) entry points take every argument by pointer, as the
 * Fortran BIND(C) routines do, and the Cp3dfft_* helpers take scalars by
 * value.  Differences, all on the caller-invisible side: the transforms run
 * on one GB300 GPU with a single-rank communicator (dims must be 1 x 1; the
 * comm handle is only checked for that), arrays may be host or device
 * pointers, and p3dfft_gb_status() / p3dfft_gb_last_error() report failures
 * (by default a failure prints a message and aborts, as MPI_Abort does in the
 * reference; p3dfft_gb_set_abort(0) makes calls return instead).
 */
#ifndef P3DFFT_GB300_DROPIN_H
#define P3DFFT_GB300_DROPIN_H

#include <stdlib.h>

#define FORT_MOD_NAME(NAME) NAME
#define FORTNAME(NAME) NAME

#ifdef SINGLE_PREC
typedef float p3dfft_real_t;
#else
typedef double p3dfft_real_t;
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* setup.F90:83 (p3dfft_setup BIND(C)) */
extern void FORT_MOD_NAME(p3dfft_setup)(int* dims, int* nx, int* ny, int* nz, int* comm, int* nxc, int* nyc,
                                        int* nzc, int* ow, int* memsize);
/* module.F90:214 */
extern void FORT_MOD_NAME(p3dfft_get_dims)(int* start, int* end, int* size, int* conf);
/* module.F90:709,719 */
extern void FORT_MOD_NAME(get_timers)(double* timers);
extern void FORT_MOD_NAME(set_timers)(void);
/* ftran.F90:469, :82 */
extern void FORT_MOD_NAME(p3dfft_ftran_r2c)(p3dfft_real_t* A, p3dfft_real_t* B, unsigned char* op);
extern void FORT_MOD_NAME(p3dfft_ftran_r2c_many)(p3dfft_real_t* A, int* dim_in, p3dfft_real_t* B, int* dim_out,
                                                 int* nv, unsigned char* op);
/* btran.F90:377, :82 */
extern void FORT_MOD_NAME(p3dfft_btran_c2r)(p3dfft_real_t* A, p3dfft_real_t* B, unsigned char* op);
extern void FORT_MOD_NAME(p3dfft_btran_c2r_many)(p3dfft_real_t* A, int* dim_in, p3dfft_real_t* B, int* dim_out,
                                                 int* nv, unsigned char* op);
/* ftran.F90:787 (a module routine of the reference without a C prototype in
 * its header): the X r2c alone, real (nx, ny, nz) -> complex (nx/2+1, ny, nz) */
extern void FORT_MOD_NAME(p3dfft_ftran_r2c_1d)(p3dfft_real_t* rXgYZ, p3dfft_real_t* cXgYZ);
/* ftran.F90:359, :321 */
extern void FORT_MOD_NAME(p3dfft_cheby)(p3dfft_real_t* A, p3dfft_real_t* B, p3dfft_real_t* Lz);
extern void FORT_MOD_NAME(p3dfft_cheby_many)(p3dfft_real_t* A, int* dim_in, p3dfft_real_t* B, int* dim_out,
                                             int* nv, p3dfft_real_t* Lz);
/* module.F90:301 */
extern void FORT_MOD_NAME(p3dfft_clean)(void);
/* module.F90:280 (single rank: taskid 0, 1 task, the comm handle given to setup) */
extern void FORT_MOD_NAME(p3dfft_get_mpi_info)(int* taskid, int* ntasks, int* comm);

/* GB300 additions: status of the last call (0 = success, negative = error),
 * its message, and the abort-on-error switch (default on).
 * p3dfft_gb_set_layout(0 | 1), called before p3dfft_setup, selects the
 * (nxhpc, nyc, nzc) output layout (0, the default) or the (nzc, nyc, nxhpc)
 * layout of the reference's STRIDE1 build (1; module.F90:245-254). */
extern int p3dfft_gb_status(void);
extern const char* p3dfft_gb_last_error(void);
extern void p3dfft_gb_set_abort(int on);
extern void p3dfft_gb_set_layout(int layout);

/* by-value helpers, as the reference's Cp3dfft_* (p3dfft.h:165-264) */
static inline void Cp3dfft_setup(int* dims, int nx, int ny, int nz, int comm, int nxc, int nyc, int nzc,
                                 int overwrite, int* memsize) {
  FORT_MOD_NAME(p3dfft_setup)(dims, &nx, &ny, &nz, &comm, &nxc, &nyc, &nzc, &overwrite, memsize);
}
static inline void Cp3dfft_clean(void) { FORT_MOD_NAME(p3dfft_clean)(); }
static inline void Cp3dfft_get_dims(int* start, int* end, int* size, int conf) {
  FORT_MOD_NAME(p3dfft_get_dims)(start, end, size, &conf);
}
static inline void Cget_timers(double* timers) { FORT_MOD_NAME(get_timers)(timers); }
static inline void Cset_timers(void) { FORT_MOD_NAME(set_timers)(); }
static inline void Cp3dfft_ftran_r2c(p3dfft_real_t* A, p3dfft_real_t* B, unsigned char* op) {
  FORT_MOD_NAME(p3dfft_ftran_r2c)(A, B, op);
}
static inline void Cp3dfft_btran_c2r(p3dfft_real_t* A, p3dfft_real_t* B, unsigned char* op) {
  FORT_MOD_NAME(p3dfft_btran_c2r)(A, B, op);
}
static inline void Cp3dfft_cheby(p3dfft_real_t* A, p3dfft_real_t* B, p3dfft_real_t Lz) {
  FORT_MOD_NAME(p3dfft_cheby)(A, B, &Lz);
}
static inline void Cp3dfft_cheby_many(p3dfft_real_t* A, int dim_in, p3dfft_real_t* B, int dim_out, int nv,
                                      p3dfft_real_t Lz) {
  FORT_MOD_NAME(p3dfft_cheby_many)(A, &dim_in, B, &dim_out, &nv, &Lz);
}
static inline void Cp3dfft_ftran_r2c_many(p3dfft_real_t* A, int dim_in, p3dfft_real_t* B, int dim_out, int nv,
                                          unsigned char* op) {
  FORT_MOD_NAME(p3dfft_ftran_r2c_many)(A, &dim_in, B, &dim_out, &nv, op);
}
static inline void Cp3dfft_btran_c2r_many(p3dfft_real_t* A, int dim_in, p3dfft_real_t* B, int dim_out, int nv,
                                          unsigned char* op) {
  FORT_MOD_NAME(p3dfft_btran_c2r_many)(A, &dim_in, B, &dim_out, &nv, op);
}

#ifdef __cplusplus
}
#endif
#endif /* P3DFFT_GB300_DROPIN_H */
