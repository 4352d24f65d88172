! wannier_gpu.f90 - Fortran drop-in for elphbolt's e-ph vertex path on one GPU.
!
! Two modules:
!  - ephg_c: the bind(C) types and interfaces of include/ephg.h (no elphbolt
!    dependency; compiles on its own with any Fortran 2008 compiler);
!  - wannier_gpu: a type that extends elphbolt's Wannier (src/wannier.f90:46-93)
!    and overrides el_wann and ph_wann with the same argument lists, so that the
!    reference's call sites (src/electron.f90:364,445,488, src/phonon.f90:210)
!    stay as they are, plus driver wrappers with the argument lists of
!    calculate_el_rta_rates (src/interactions.f90:2958) and
!    calculate_ph_rta_rates (:2723), which replace the gkRp / 'g' / 'X' (and
!    gReq / 'g' / 'Y') passes and their files by one library call each.
!
! Build: compile with the elphbolt sources (it uses the modules precision,
! misc, crystal_module, electron_module, numerics_module and wannier_module)
! and link libephg.so.  A caller declares
!     type(wannier_gpu_t) :: wann
! where it declared type(Wannier), calls wann%read(num) as before, and then
! wann%upload(crys), which reads epmatwp1 once more and hands every array to
! ephg_create (the library keeps them resident on the device; gwann is a
! private module variable of wannier_module, so it is read from the file).

module ephg_c
  use iso_c_binding
  implicit none

  integer(c_int), parameter :: EPHG_OK = 0
  integer(c_int64_t), parameter :: EPHG_PREC_FP64 = 0, EPHG_PREC_SPLIT_TF32 = 1
  integer(c_int64_t), parameter :: EPHG_DELTA_GAUSSIAN = 0, EPHG_DELTA_TRIANGLE = 1, &
       EPHG_DELTA_TETRA = 2
  integer(c_int64_t), parameter :: EPHG_WANNSPACE_EL = 0, EPHG_WANNSPACE_PH = 1
  integer(c_int64_t), parameter :: EPHG_DEGAVG_REFERENCE = 0, EPHG_DEGAVG_MEAN = 1

  type, bind(C) :: ephg_wannier_desc
     integer(c_int64_t) :: numwannbands, numbranches, nwsk, nwsq, nwsg, numatoms
     integer(c_int64_t) :: coarse_qmesh(3)
     type(c_ptr) :: lattvecs, basis, masses
     type(c_ptr) :: rcells_k, rcells_q, rcells_g, elwsdeg, phwsdeg, gwsdeg
     type(c_ptr) :: Hwann, Dphwann, gwann
  end type ephg_wannier_desc

  type, bind(C) :: ephg_rate_request
     integer(c_int64_t) :: mesh(3)
     real(c_double) :: enref, fsthick, chempot, T
     integer(c_int64_t) :: delta_kind
     real(c_double) :: sigma
     integer(c_int64_t) :: precision
  end type ephg_rate_request

  type, bind(C) :: ephg_rate_stats
     integer(c_int64_t) :: nwv, nstates_inwindow, nstates, vertices, pairs, kernel_launches
     real(c_double) :: ms_setup, ms_stage_a, ms_stage_bc, ms_total, stage_b_gflop, stage_a_gflop, &
          ms_gemm_a, ms_gemm_b
     integer(c_int64_t) :: gemm_a_launches, gemm_b_launches
  end type ephg_rate_stats

  type, bind(C) :: ephg_batch_opts
     integer(c_int64_t) :: nslots, hbm_budget_bytes, grouped
  end type ephg_batch_opts

  type, bind(C) :: ephg_batch_stats
     integer(c_int64_t) :: requests, failed, vertices
     real(c_double) :: wall_ms, vertices_per_s
     integer(c_int64_t) :: group_launches, group_problems, group_tiles, max_group, retried_alone, &
          peak_workspace_bytes
  end type ephg_batch_stats

  type, bind(C) :: ephg_server_stats
     integer(c_int64_t) :: submitted, completed, failed, rejected, vertices
     real(c_double) :: p50_ms, p99_ms, max_ms, mean_ms, wall_s, vertices_per_s
     integer(c_int64_t) :: peak_device_bytes, merged
  end type ephg_server_stats

  interface
     integer(c_int) function ephg_create(desc, h) bind(C, name="ephg_create")
       import :: c_int, c_ptr, ephg_wannier_desc
       type(ephg_wannier_desc), intent(in) :: desc
       type(c_ptr), intent(out) :: h
     end function ephg_create

     integer(c_int) function ephg_destroy(h) bind(C, name="ephg_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: h
     end function ephg_destroy

     type(c_ptr) function ephg_last_error() bind(C, name="ephg_last_error")
       import :: c_ptr
     end function ephg_last_error

     integer(c_int) function ephg_device_count() bind(C, name="ephg_device_count")
       import :: c_int
     end function ephg_device_count

     integer(c_int) function ephg_trim_memory() bind(C, name="ephg_trim_memory")
       !! return the library pool's unused device memory to the driver
       import :: c_int
     end function ephg_trim_memory

     integer(c_int) function ephg_set_polar(h, epsilon, born) bind(C, name="ephg_set_polar")
       import :: c_int, c_ptr
       type(c_ptr), value :: h, epsilon, born
     end function ephg_set_polar

     integer(c_int) function ephg_crystal_symmetry(lattvecs, natoms, basis, atomtypes, symprec, &
          maxops, nops, rotations, translations) bind(C, name="ephg_crystal_symmetry")
       import :: c_int, c_ptr, c_int64_t, c_double
       type(c_ptr), value :: lattvecs, basis, atomtypes, nops, rotations, translations
       integer(c_int64_t), value :: natoms, maxops
       real(c_double), value :: symprec
     end function ephg_crystal_symmetry

     integer(c_int) function ephg_set_symmetry(h, nsymm, rotations) bind(C, name="ephg_set_symmetry")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h, rotations
       integer(c_int64_t), value :: nsymm
     end function ephg_set_symmetry

     integer(c_int) function ephg_irred_wedge(lattvecs, nsymm, rotations, mesh, nk, indexlist, &
          nirred, indexlist_irred, nequiv, fbz2ibz) bind(C, name="ephg_irred_wedge")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: lattvecs, rotations, mesh, indexlist, nirred, indexlist_irred, &
            nequiv, fbz2ibz
       integer(c_int64_t), value :: nsymm, nk
     end function ephg_irred_wedge

     integer(c_int) function ephg_el_wann(h, nk, kvecs, energies, velocities, evecs, scissor) &
          bind(C, name="ephg_el_wann")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h, kvecs, energies, velocities, evecs, scissor
       integer(c_int64_t), value :: nk
     end function ephg_el_wann

     integer(c_int) function ephg_ph_wann(h, nq, qvecs, energies, evecs, velocities) &
          bind(C, name="ephg_ph_wann")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h, qvecs, energies, evecs, velocities
       integer(c_int64_t), value :: nq
     end function ephg_ph_wann

     integer(c_int) function ephg_gkRp(h, nk, kvecs, gmixed) bind(C, name="ephg_gkRp")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h, kvecs, gmixed
       integer(c_int64_t), value :: nk
     end function ephg_gkRp

     integer(c_int) function ephg_gReq(h, nq, qvecs, gmixed) bind(C, name="ephg_gReq")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h, qvecs, gmixed
       integer(c_int64_t), value :: nq
     end function ephg_gReq

     integer(c_int) function ephg_g2(h, wannspace, nv, kvecs, qvecs, el_evec_k, el_evec_kp, &
          ph_evec_q, ph_en, ngm, gmixed, gm_index, g2_out) bind(C, name="ephg_g2")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h, kvecs, qvecs, el_evec_k, el_evec_kp, ph_evec_q, ph_en, gmixed, &
            gm_index, g2_out
       integer(c_int64_t), value :: wannspace, nv, ngm
     end function ephg_g2

     integer(c_int) function ephg_kq_index(h, mesh, nk, k_idx, nkp, kp_idx, q_idx) &
          bind(C, name="ephg_kq_index")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h, mesh, k_idx, kp_idx, q_idx
       integer(c_int64_t), value :: nk, nkp
     end function ephg_kq_index

     integer(c_int) function ephg_el_rates(h, req, rates, indexlist, stats, g2, xplus, xminus, cap) &
          bind(C, name="ephg_el_rates")
       import :: c_int, c_ptr, c_int64_t, ephg_rate_request
       type(c_ptr), value :: h, rates, indexlist, stats, g2, xplus, xminus
       type(ephg_rate_request), intent(in) :: req
       integer(c_int64_t), value :: cap
     end function ephg_el_rates

     integer(c_int) function ephg_el_rates_sets(h, nsets, reqs, rates, indexlist, stats) &
          bind(C, name="ephg_el_rates_sets")
       !! nsets (<= 8) requests equal but for T, sigma and chempot: one contraction;
       !! reqs: nsets requests; rates: an array of nsets C pointers (c_loc of each (N,nw) array)
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h, reqs, rates, indexlist, stats
       integer(c_int64_t), value :: nsets
     end function ephg_el_rates_sets

     integer(c_int) function ephg_ph_rates(h, req, spindeg, rates_phe, el_rates, indexlist, stats, &
          g2, y, cap) bind(C, name="ephg_ph_rates")
       import :: c_int, c_ptr, c_int64_t, ephg_rate_request
       type(c_ptr), value :: h, rates_phe, el_rates, indexlist, stats, g2, y
       type(ephg_rate_request), intent(in) :: req
       integer(c_int64_t), value :: spindeg, cap
     end function ephg_ph_rates

     integer(c_int) function ephg_g2_average_degenerate(h, req, mode, thres, nv, g2) &
          bind(C, name="ephg_g2_average_degenerate")
       !! mode 0: the reference's in-place loops (wannier.f90:1332-1384); 1: gauge-invariant means
       import :: c_int, c_ptr, c_int64_t, c_double, ephg_rate_request
       type(c_ptr), value :: h, g2
       type(ephg_rate_request), intent(in) :: req
       integer(c_int64_t), value :: mode, nv
       real(c_double), value :: thres
     end function ephg_g2_average_degenerate

     integer(c_int) function ephg_el_wann_noalloc(h, nk, kvecs, energies, evecs) &
          bind(C, name="ephg_el_wann_noalloc")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: h, kvecs, energies, evecs
       integer(c_int64_t), value :: nk
     end function ephg_el_wann_noalloc

     integer(c_int) function ephg_el_rates_batch(n, crystals, reqs, rates, indexlists, stats, status, &
          opts, bstats) bind(C, name="ephg_el_rates_batch")
       !! crystals, rates, indexlists: arrays of n C pointers; reqs: n requests
       import :: c_int, c_ptr, c_int64_t, ephg_batch_opts
       integer(c_int64_t), value :: n
       type(c_ptr), value :: crystals, reqs, rates, indexlists, stats, status, bstats
       type(ephg_batch_opts), intent(in) :: opts
     end function ephg_el_rates_batch

     integer(c_int) function ephg_server_create(crystals, ncrystals, hbm_budget_bytes, nslots, srv) &
          bind(C, name="ephg_server_create")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: crystals
       integer(c_int), value :: ncrystals, nslots
       integer(c_int64_t), value :: hbm_budget_bytes
       type(c_ptr), intent(out) :: srv
     end function ephg_server_create

     integer(c_int) function ephg_server_destroy(srv) bind(C, name="ephg_server_destroy")
       import :: c_int, c_ptr
       type(c_ptr), value :: srv
     end function ephg_server_destroy

     integer(c_int) function ephg_submit(srv, crystal, req, ticket) bind(C, name="ephg_submit")
       import :: c_int, c_ptr, c_int64_t, ephg_rate_request
       type(c_ptr), value :: srv
       integer(c_int), value :: crystal
       type(ephg_rate_request), intent(in) :: req
       integer(c_int64_t), intent(out) :: ticket
     end function ephg_submit

     integer(c_int) function ephg_poll(srv, ticket, state) bind(C, name="ephg_poll")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: srv
       integer(c_int64_t), value :: ticket
       integer(c_int), intent(out) :: state
     end function ephg_poll

     integer(c_int) function ephg_wait(srv, ticket, rates, indexlist, stats, latency_ms) &
          bind(C, name="ephg_wait")
       import :: c_int, c_ptr, c_int64_t
       type(c_ptr), value :: srv, rates, indexlist, stats, latency_ms
       integer(c_int64_t), value :: ticket
     end function ephg_wait

     integer(c_int) function ephg_server_set_merge(srv, max_sets) bind(C, name="ephg_server_set_merge")
       import :: c_int, c_ptr
       type(c_ptr), value :: srv
       integer(c_int), value :: max_sets
     end function ephg_server_set_merge

     integer(c_int) function ephg_server_stats_get(srv, st) bind(C, name="ephg_server_stats_get")
       import :: c_int, c_ptr, ephg_server_stats
       type(c_ptr), value :: srv
       type(ephg_server_stats), intent(out) :: st
     end function ephg_server_stats_get

     integer(c_size_t) function c_strlen(s) bind(C, name="strlen")
       import :: c_size_t, c_ptr
       type(c_ptr), value :: s
     end function c_strlen
  end interface

contains

  function ephg_message() result(msg)
    !! ephg_last_error() as a Fortran string.
    character(len=:), allocatable :: msg
    type(c_ptr) :: p
    character(kind=c_char), pointer :: chars(:)
    integer :: i, n
    p = ephg_last_error()
    if(.not. c_associated(p)) then
       msg = ""
       return
    end if
    n = int(c_strlen(p))
    call c_f_pointer(p, chars, [n])
    allocate(character(len=n) :: msg)
    do i = 1, n
       msg(i:i) = chars(i)
    end do
  end function ephg_message
end module ephg_c

module wannier_gpu
  use iso_c_binding
  use ephg_c
  use precision, only: r64, i64
  use misc, only: exit_with_message
  use crystal_module, only: crystal
  use wannier_module, only: Wannier
  use electron_module, only: electron
  use numerics_module, only: numerics
  implicit none

  private
  public :: wannier_gpu_t, calculate_el_rta_rates_gpu, calculate_ph_rta_rates_gpu

  type, extends(Wannier) :: wannier_gpu_t
     !! elphbolt's Wannier data plus the handle of its device-resident copy.
     type(c_ptr) :: h = c_null_ptr
     integer(i64) :: precision = EPHG_PREC_SPLIT_TF32
     !! precision of the rate drivers: EPHG_PREC_FP64 or EPHG_PREC_SPLIT_TF32
   contains
     procedure :: upload
     procedure :: el_wann => el_wann_gpu
     procedure :: ph_wann => ph_wann_gpu
     procedure :: deallocate_wannier => deallocate_wannier_gpu
  end type wannier_gpu_t

contains

  subroutine check(rc, where)
    integer(c_int), intent(in) :: rc
    character(len=*), intent(in) :: where
    if(rc /= EPHG_OK) call exit_with_message(where//": "//ephg_message())
  end subroutine check

  subroutine upload(self, crys, epmatwp_file)
    !! After self%read(num): hand the Wannier data and the crystal to the
    !! library (ephg_create); polar crystals also get epsilon and the Born
    !! charges (ephg_set_polar).  One image holds all of g(Re,Rp), read again
    !! from epmatwp_file (default 'epmatwp1', as read_EPW_Wannier reads it).
    class(wannier_gpu_t), intent(inout) :: self
    type(crystal), intent(in), target :: crys
    character(len=*), intent(in), optional :: epmatwp_file
    type(ephg_wannier_desc) :: d
    complex(r64), allocatable, target :: g(:, :, :, :, :)
    integer(i64), allocatable, target :: rk(:, :), rq(:, :), rg(:, :), dk(:), dq(:), dg(:)
    complex(r64), allocatable, target :: H(:, :, :), Dm(:, :, :)
    real(r64), allocatable, target :: lat(:, :), bas(:, :), mas(:), eps(:, :), born(:, :, :)
    integer :: u

    allocate(g(self%numwannbands, self%numwannbands, self%nwsk, self%numbranches, self%nwsg))
    if(present(epmatwp_file)) then
       open(newunit = u, file = epmatwp_file, status = 'old', access = 'stream')
    else
       open(newunit = u, file = 'epmatwp1', status = 'old', access = 'stream')
    end if
    read(u) g
    close(u)
    ! target copies of the (allocatable, partly coarray) fields
    rk = self%rcells_k
    rq = self%rcells_q
    rg = self%rcells_g(:, :)
    dk = self%elwsdeg
    dq = self%phwsdeg
    dg = self%gwsdeg(:)
    H = self%Hwann
    Dm = self%Dphwann
    lat = crys%lattvecs
    bas = crys%basis
    mas = crys%masses(crys%atomtypes)

    d%numwannbands = self%numwannbands
    d%numbranches = self%numbranches
    d%nwsk = self%nwsk
    d%nwsq = self%nwsq
    d%nwsg = self%nwsg
    d%numatoms = crys%numatoms
    d%coarse_qmesh = self%coarse_qmesh
    d%lattvecs = c_loc(lat)
    d%basis = c_loc(bas)
    d%masses = c_loc(mas)
    d%rcells_k = c_loc(rk)
    d%rcells_q = c_loc(rq)
    d%rcells_g = c_loc(rg)
    d%elwsdeg = c_loc(dk)
    d%phwsdeg = c_loc(dq)
    d%gwsdeg = c_loc(dg)
    d%Hwann = c_loc(H)
    d%Dphwann = c_loc(Dm)
    d%gwann = c_loc(g)
    call check(ephg_create(d, self%h), "ephg_create")
    if(crys%polar) then
       eps = crys%epsilon
       born = crys%born
       call check(ephg_set_polar(self%h, c_loc(eps), c_loc(born)), "ephg_set_polar")
    end if
  end subroutine upload

  subroutine el_wann_gpu(self, crys, nk, kvecs, energies, velocities, evecs, scissor)
    !! el_wann (src/wannier.f90:430-524) on the device: same arguments.
    class(wannier_gpu_t), intent(in) :: self
    type(crystal), intent(in) :: crys
    integer(i64), intent(in) :: nk
    real(r64), intent(in) :: kvecs(nk, 3)
    real(r64), intent(out) :: energies(nk, self%numwannbands)
    real(r64), optional, intent(out) :: velocities(nk, self%numwannbands, 3)
    complex(r64), optional, intent(out) :: evecs(nk, self%numwannbands, self%numwannbands)
    real(r64), optional, intent(in) :: scissor(self%numwannbands)
    real(r64), allocatable, target :: k(:, :), e(:, :), v(:, :, :), sc(:)
    complex(r64), allocatable, target :: ev(:, :, :)
    type(c_ptr) :: pv, pev, psc

    if(present(velocities) .and. .not. present(evecs)) &
         call exit_with_message("In el_wann, velocity is present but not eigenvecs.")
    k = kvecs
    allocate(e(nk, self%numwannbands))
    pv = c_null_ptr
    pev = c_null_ptr
    psc = c_null_ptr
    if(present(velocities)) then
       allocate(v(nk, self%numwannbands, 3))
       pv = c_loc(v)
    end if
    if(present(evecs)) then
       allocate(ev(nk, self%numwannbands, self%numwannbands))
       pev = c_loc(ev)
    end if
    if(present(scissor)) then
       sc = scissor
       psc = c_loc(sc)
    end if
    call check(ephg_el_wann(self%h, nk, c_loc(k), c_loc(e), pv, pev, psc), "ephg_el_wann")
    energies = e
    if(present(velocities)) velocities = v
    if(present(evecs)) evecs = ev
  end subroutine el_wann_gpu

  subroutine ph_wann_gpu(self, crys, nq, qvecs, energies, evecs, velocities)
    !! ph_wann (src/wannier.f90:585-782) on the device: same arguments; the
    !! polar term is on when upload found crys%polar.
    class(wannier_gpu_t), intent(in) :: self
    type(crystal), intent(in) :: crys
    integer(i64), intent(in) :: nq
    real(r64), intent(in) :: qvecs(nq, 3)
    real(r64), intent(out) :: energies(nq, self%numbranches)
    real(r64), optional, intent(out) :: velocities(nq, self%numbranches, 3)
    complex(r64), intent(out), optional :: evecs(nq, self%numbranches, self%numbranches)
    real(r64), allocatable, target :: q(:, :), e(:, :), v(:, :, :)
    complex(r64), allocatable, target :: ev(:, :, :)
    type(c_ptr) :: pv, pev

    if(present(velocities) .and. .not. present(evecs)) &
         call exit_with_message("In ph_wann, velocity is present but not eigenvecs.")
    q = qvecs
    allocate(e(nq, self%numbranches))
    pv = c_null_ptr
    pev = c_null_ptr
    if(present(velocities)) then
       allocate(v(nq, self%numbranches, 3))
       pv = c_loc(v)
    end if
    if(present(evecs)) then
       allocate(ev(nq, self%numbranches, self%numbranches))
       pev = c_loc(ev)
    end if
    call check(ephg_ph_wann(self%h, nq, c_loc(q), c_loc(e), pev, pv), "ephg_ph_wann")
    energies = e
    if(present(velocities)) velocities = v
    if(present(evecs)) evecs = ev
  end subroutine ph_wann_gpu

  subroutine deallocate_wannier_gpu(self, num)
    !! deallocate_wannier, plus the device copy.
    class(wannier_gpu_t), intent(inout) :: self
    type(numerics), intent(in) :: num
    integer(c_int) :: rc
    if(c_associated(self%h)) then
       rc = ephg_destroy(self%h)
       self%h = c_null_ptr
    end if
    call self%Wannier%deallocate_wannier(num)
  end subroutine deallocate_wannier_gpu

  function rate_request(el, crys, num, precision) result(r)
    !! The settings the ibzk / ibzq drivers read: the electron mesh (= phonon
    !! mesh, mesh_ref = 1), window, chemical potential, temperature and the
    !! delta method (num%tetrahedra: tetrahedron, else triangle).
    type(electron), intent(in) :: el
    type(crystal), intent(in) :: crys
    type(numerics), intent(in) :: num
    integer(i64), intent(in) :: precision
    type(ephg_rate_request) :: r
    r%mesh = el%wvmesh
    r%enref = el%enref
    r%fsthick = el%fsthick
    r%chempot = el%chempot
    r%T = crys%T
    if(num%tetrahedra) then
       r%delta_kind = EPHG_DELTA_TETRA
    else
       r%delta_kind = EPHG_DELTA_TRIANGLE
    end if
    r%sigma = 0.0_r64
    r%precision = precision
  end function rate_request

  subroutine calculate_el_rta_rates_gpu(wann, rta_rates_eph, num, crys, el)
    !! calculate_gkRp + calculate_eph_interaction_ibzk('g') + ('X') +
    !! the e-ph part of calculate_el_rta_rates (src/interactions.f90:1632,
    !! 2095, 2958) in one ephg_el_rates call, with no files: rta_rates_eph
    !! (nwv_irred, nw) over the window blocks in indexlist_irred order.  With
    !! a point group, call ephg_set_symmetry(wann%h, sym%nsymm,
    !! c_loc(sym%rotations_orig)) once first.
    class(wannier_gpu_t), intent(in) :: wann
    real(r64), allocatable, intent(out) :: rta_rates_eph(:, :)
    type(numerics), intent(in) :: num
    type(crystal), intent(in) :: crys
    type(electron), intent(in) :: el
    type(ephg_rate_request) :: r
    type(ephg_rate_stats), target :: st
    real(r64), allocatable, target :: rates(:, :)
    integer(i64), allocatable, target :: idx(:)
    integer(i64) :: nk

    r = rate_request(el, crys, num, wann%precision)
    nk = product(el%wvmesh)
    allocate(rates(nk, wann%numwannbands), idx(nk))
    call check(ephg_el_rates(wann%h, r, c_loc(rates), c_loc(idx), c_loc(st), c_null_ptr, &
         c_null_ptr, c_null_ptr, 0_c_int64_t), "ephg_el_rates")
    allocate(rta_rates_eph(st%nwv, wann%numwannbands))
    rta_rates_eph = rates(1:st%nwv, :)
  end subroutine calculate_el_rta_rates_gpu

  subroutine calculate_ph_rta_rates_gpu(wann, rta_rates_phe, num, crys, el)
    !! calculate_gReq + calculate_eph_interaction_ibzq('g') + ('Y') (or
    !! calculate_Y_OTF) + the ph-e part of calculate_ph_rta_rates
    !! (src/interactions.f90:1603, 1673, 1932, 2723) in one ephg_ph_rates
    !! call: rta_rates_phe (nq, nb) over every q of the mesh, spindeg el%spindeg.
    class(wannier_gpu_t), intent(in) :: wann
    real(r64), allocatable, intent(out) :: rta_rates_phe(:, :)
    type(numerics), intent(in) :: num
    type(crystal), intent(in) :: crys
    type(electron), intent(in) :: el
    type(ephg_rate_request) :: r
    real(r64), allocatable, target :: rates(:, :)
    integer(i64) :: nq

    r = rate_request(el, crys, num, wann%precision)
    nq = product(el%wvmesh)
    allocate(rates(nq, wann%numbranches))
    call check(ephg_ph_rates(wann%h, r, int(el%spindeg, c_int64_t), c_loc(rates), c_null_ptr, &
         c_null_ptr, c_null_ptr, c_null_ptr, c_null_ptr, 0_c_int64_t), "ephg_ph_rates")
    call move_alloc(rates, rta_rates_phe)
  end subroutine calculate_ph_rta_rates_gpu
end module wannier_gpu
