! Fortran module p3dfft for the GB300 P3DFFT library.
!
! The reference's public Fortran surface (build/module.F90:92-106,178-186:
! p3dfft_type, r8, i8, timers and the p3dfft_* routines; build/setup.F90:107-141
! for the optional arguments of p3dfft_setup; build/wrap.F90:82-150 for the
! external ftran_r2c / btran_c2r wrappers) bound with ISO_C_BINDING to the C
! symbols of libp3dfft.so (or libp3dfft_single.so when compiled with
! -DSINGLE_PREC).  Build and link, e.g.:
!
!   gfortran -cpp -c p3dfft.F90
!   gfortran app.f90 p3dfft.o -L<repo>/p3dfft_gb300/_lib -lp3dfft -Wl,-rpath,<repo>/p3dfft_gb300/_lib
!
! The processor grid must be 1 x 1 and mpi_comm_in is only recorded (one GPU,
! single-rank communicator).  Errors print and stop the program as in the
! reference.
module p3dfft
  use iso_c_binding
  implicit none
  private

#ifdef SINGLE_PREC
  integer, parameter, public :: p3dfft_type = c_float
#else
  integer, parameter, public :: p3dfft_type = c_double
#endif
  integer, parameter, public :: r8 = kind(1.0d0)
  integer, parameter, public :: i8 = selected_int_kind(18)
  ! the 12 stage timers, refreshed by get_timers (build/module.F90:106)
  real(r8), save, public :: timers(12) = 0.0_r8

  public :: p3dfft_setup, p3dfft_get_dims, p3dfft_get_mpi_info
  public :: p3dfft_ftran_r2c, p3dfft_btran_c2r, p3dfft_cheby, p3dfft_ftran_r2c_1d
  public :: p3dfft_ftran_r2c_many, p3dfft_btran_c2r_many, p3dfft_cheby_many
  public :: p3dfft_clean, get_timers, set_timers

  interface
    subroutine c_setup(dims, nx, ny, nz, comm, nxc, nyc, nzc, ow, memsize) bind(C, name='p3dfft_setup')
      import :: c_int
      integer(c_int) :: dims(2), nx, ny, nz, comm, nxc, nyc, nzc, ow, memsize(3)
    end subroutine c_setup
    subroutine c_get_dims(istart, iend, isize, conf) bind(C, name='p3dfft_get_dims')
      import :: c_int
      integer(c_int) :: istart(3), iend(3), isize(3), conf
    end subroutine c_get_dims
    subroutine c_get_mpi_info(taskid, ntasks, comm) bind(C, name='p3dfft_get_mpi_info')
      import :: c_int
      integer(c_int) :: taskid, ntasks, comm
    end subroutine c_get_mpi_info
    subroutine c_ftran(a, b, op) bind(C, name='p3dfft_ftran_r2c')
      import :: c_char, p3dfft_type
      real(p3dfft_type) :: a(*)
      complex(p3dfft_type) :: b(*)
      character(kind=c_char) :: op(*)
    end subroutine c_ftran
    subroutine c_btran(a, b, op) bind(C, name='p3dfft_btran_c2r')
      import :: c_char, p3dfft_type
      complex(p3dfft_type) :: a(*)
      real(p3dfft_type) :: b(*)
      character(kind=c_char) :: op(*)
    end subroutine c_btran
    subroutine c_ftran_many(a, dim_in, b, dim_out, nv, op) bind(C, name='p3dfft_ftran_r2c_many')
      import :: c_char, c_int, p3dfft_type
      real(p3dfft_type) :: a(*)
      integer(c_int) :: dim_in, dim_out, nv
      complex(p3dfft_type) :: b(*)
      character(kind=c_char) :: op(*)
    end subroutine c_ftran_many
    subroutine c_btran_many(a, dim_in, b, dim_out, nv, op) bind(C, name='p3dfft_btran_c2r_many')
      import :: c_char, c_int, p3dfft_type
      complex(p3dfft_type) :: a(*)
      integer(c_int) :: dim_in, dim_out, nv
      real(p3dfft_type) :: b(*)
      character(kind=c_char) :: op(*)
    end subroutine c_btran_many
    subroutine c_ftran_1d(a, b) bind(C, name='p3dfft_ftran_r2c_1d')
      import :: p3dfft_type
      real(p3dfft_type) :: a(*)
      real(p3dfft_type) :: b(*)
    end subroutine c_ftran_1d
    subroutine c_cheby(a, b, lz) bind(C, name='p3dfft_cheby')
      import :: p3dfft_type
      real(p3dfft_type) :: a(*)
      complex(p3dfft_type) :: b(*)
      real(p3dfft_type) :: lz
    end subroutine c_cheby
    subroutine c_cheby_many(a, dim_in, b, dim_out, nv, lz) bind(C, name='p3dfft_cheby_many')
      import :: c_int, p3dfft_type
      real(p3dfft_type) :: a(*)
      integer(c_int) :: dim_in, dim_out, nv
      complex(p3dfft_type) :: b(*)
      real(p3dfft_type) :: lz
    end subroutine c_cheby_many
    subroutine c_clean() bind(C, name='p3dfft_clean')
    end subroutine c_clean
    subroutine c_get_timers(t) bind(C, name='get_timers')
      import :: c_double
      real(c_double) :: t(12)
    end subroutine c_get_timers
    subroutine c_set_timers() bind(C, name='set_timers')
    end subroutine c_set_timers
  end interface

contains

  ! setup.F90:107-141: overwrite defaults to .true.; nxcut etc. default to n
  subroutine p3dfft_setup(dims, nx, ny, nz, mpi_comm_in, nxcut, nycut, nzcut, overwrite, memsize)
    integer, intent(in) :: dims(2), nx, ny, nz, mpi_comm_in
    integer, intent(in), optional :: nxcut, nycut, nzcut
    logical, intent(in), optional :: overwrite
    integer, intent(out), optional :: memsize(3)
    integer(c_int) :: d(2), cnx, cny, cnz, comm, cx, cy, cz, ow, ms(3)
    d = int(dims, c_int)
    cnx = nx
    cny = ny
    cnz = nz
    comm = mpi_comm_in
    cx = nx
    cy = ny
    cz = nz
    if (present(nxcut)) cx = nxcut
    if (present(nycut)) cy = nycut
    if (present(nzcut)) cz = nzcut
    ow = 1
    if (present(overwrite)) then
      if (.not. overwrite) ow = 0
    end if
    ms = 0
    call c_setup(d, cnx, cny, cnz, comm, cx, cy, cz, ow, ms)
    if (present(memsize)) memsize = int(ms)
    timers = 0.0_r8
  end subroutine p3dfft_setup

  subroutine p3dfft_get_dims(istart, iend, isize, conf)
    integer, intent(out) :: istart(3), iend(3), isize(3)
    integer, intent(in) :: conf
    integer(c_int) :: s(3), e(3), z(3), c
    c = conf
    call c_get_dims(s, e, z, c)
    istart = int(s)
    iend = int(e)
    isize = int(z)
  end subroutine p3dfft_get_dims

  subroutine p3dfft_get_mpi_info(taskid, ntasks, comm)
    integer, intent(out) :: taskid, ntasks, comm
    integer(c_int) :: t, n, c
    call c_get_mpi_info(t, n, c)
    taskid = t
    ntasks = n
    comm = c
  end subroutine p3dfft_get_mpi_info

  subroutine p3dfft_ftran_r2c(XgYZ, XYZg, op)
    real(p3dfft_type), intent(in) :: XgYZ(*)
    complex(p3dfft_type), intent(inout) :: XYZg(*)
    character(len=3), intent(in) :: op
    call c_ftran(XgYZ, XYZg, op)
  end subroutine p3dfft_ftran_r2c

  subroutine p3dfft_btran_c2r(XYZg, XgYZ, op)
    complex(p3dfft_type), intent(in) :: XYZg(*)
    real(p3dfft_type), intent(inout) :: XgYZ(*)
    character(len=3), intent(in) :: op
    call c_btran(XYZg, XgYZ, op)
  end subroutine p3dfft_btran_c2r

  subroutine p3dfft_ftran_r2c_many(XgYZ, dim_in, XYZg, dim_out, nv, op)
    integer, intent(in) :: dim_in, dim_out, nv
    real(p3dfft_type), intent(in) :: XgYZ(*)
    complex(p3dfft_type), intent(inout) :: XYZg(*)
    character(len=3), intent(in) :: op
    integer(c_int) :: di, dout, n
    di = dim_in
    dout = dim_out
    n = nv
    call c_ftran_many(XgYZ, di, XYZg, dout, n, op)
  end subroutine p3dfft_ftran_r2c_many

  subroutine p3dfft_btran_c2r_many(XYZg, dim_in, XgYZ, dim_out, nv, op)
    integer, intent(in) :: dim_in, dim_out, nv
    complex(p3dfft_type), intent(in) :: XYZg(*)
    real(p3dfft_type), intent(inout) :: XgYZ(*)
    character(len=3), intent(in) :: op
    integer(c_int) :: di, dout, n
    di = dim_in
    dout = dim_out
    n = nv
    call c_btran_many(XYZg, di, XgYZ, dout, n, op)
  end subroutine p3dfft_btran_c2r_many

  ! ftran.F90:383-464: 'ffc' transform, scaling and the derivative recurrence
  ! ftran.F90:787-814: the X r2c alone; cXgYZ holds nx/2+1 complexes per line
  subroutine p3dfft_ftran_r2c_1d(rXgYZ, cXgYZ)
    real(p3dfft_type), intent(in) :: rXgYZ(*)
    real(p3dfft_type), intent(inout) :: cXgYZ(*)
    call c_ftran_1d(rXgYZ, cXgYZ)
  end subroutine p3dfft_ftran_r2c_1d

  subroutine p3dfft_cheby(XgYZ, XYZg, Lz)
    real(p3dfft_type), intent(in) :: XgYZ(*)
    complex(p3dfft_type), intent(inout) :: XYZg(*)
    real(p3dfft_type), intent(in) :: Lz
    real(p3dfft_type) :: l
    l = Lz
    call c_cheby(XgYZ, XYZg, l)
  end subroutine p3dfft_cheby

  subroutine p3dfft_cheby_many(XgYZ, dim_in, XYZg, dim_out, nv, Lz)
    integer, intent(in) :: dim_in, dim_out, nv
    real(p3dfft_type), intent(in) :: XgYZ(*)
    complex(p3dfft_type), intent(inout) :: XYZg(*)
    real(p3dfft_type), intent(in) :: Lz
    integer(c_int) :: di, dout, n
    real(p3dfft_type) :: l
    di = dim_in
    dout = dim_out
    n = nv
    l = Lz
    call c_cheby_many(XgYZ, di, XYZg, dout, n, l)
  end subroutine p3dfft_cheby_many

  subroutine p3dfft_clean()
    call c_clean()
  end subroutine p3dfft_clean

  subroutine get_timers(t)
    real(r8), intent(out) :: t(12)
    real(c_double) :: ct(12)
    call c_get_timers(ct)
    t = ct
    timers = ct
  end subroutine get_timers

  subroutine set_timers()
    call c_set_timers()
    timers = 0.0_r8
  end subroutine set_timers

end module p3dfft

! wrap.F90:82-150: external wrappers taking the same array for input and
! output (in-place use, sized by memsize)
subroutine ftran_r2c(IN, OUT, op)
  use p3dfft
  real(p3dfft_type), target :: IN(1, 1, *)
  complex(p3dfft_type), target :: OUT(1, 1, *)
  character(len=3) op
  call p3dfft_ftran_r2c(IN, OUT, op)
end subroutine ftran_r2c

subroutine btran_c2r(IN, OUT, op)
  use p3dfft
  complex(p3dfft_type), target :: IN(1, 1, *)
  real(p3dfft_type), target :: OUT(1, 1, *)
  character(len=3) op
  call p3dfft_btran_c2r(IN, OUT, op)
end subroutine btran_c2r

subroutine ftran_r2c_many(IN, dim_in, OUT, dim_out, nv, op)
  use p3dfft
  integer dim_in, dim_out, nv
  real(p3dfft_type), target :: IN(dim_in, nv)
  complex(p3dfft_type), target :: OUT(dim_out, nv)
  character(len=3) op
  call p3dfft_ftran_r2c_many(IN, dim_in, OUT, dim_out, nv, op)
end subroutine ftran_r2c_many

subroutine btran_c2r_many(IN, dim_in, OUT, dim_out, nv, op)
  use p3dfft
  integer dim_in, dim_out, nv
  complex(p3dfft_type), target :: IN(dim_in, nv)
  real(p3dfft_type), target :: OUT(dim_out, nv)
  character(len=3) op
  call p3dfft_btran_c2r_many(IN, dim_in, OUT, dim_out, nv, op)
end subroutine btran_c2r_many
