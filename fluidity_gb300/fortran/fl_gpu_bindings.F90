!    fl_gpu_bindings.F90 -- ISO_C_BINDING interface to libfluidity_gb300.so.
!
!    The Fortran side of the drop-in boundary: explicit interfaces to the
!    C-ABI declared in include/fluidity_gb300.h, plus wrappers that take
!    Fluidity's own types (csr_matrix, scalar_field, vector_field, mesh_type)
!    and call the GPU entry points with c_loc() pointers to the arrays those
!    types already own.  The wrappers keep the argument meaning of the routines
!    they stand in for:
!
!      gpu_assemble_advection_diffusion_cg  -> assemble_advection_diffusion_cg
!                                    (assemble/Advection_Diffusion_CG.F90:228)
!      gpu_petsc_solve_scalar       -> petsc_solve_scalar (femtools/Solvers.F90:111)
!
!    Status handling follows the reference: usage errors abort with FLAbort
!    (include/fdebug.h:56), solver divergence is returned as a negative
!    KSPConvergedReason for ConvergenceCheck (femtools/Solvers.F90:1369).
!
!    Not compiled in this repository's build (no Fortran compiler is
!    available); it is compiled into Fluidity's femtools library by the
!    integration recipe of INTEGRATION.md.
#include "fdebug.h"
module fl_gpu_bindings
  use iso_c_binding
  implicit none
  private

  public :: fl_mesh_desc, fl_advdif_params, fl_fields, fl_solver_opts, fl_solve_report
  public :: fl_gpu_mesh_register, fl_gpu_mesh_destroy, fl_gpu_mesh_info, &
            fl_gpu_sparsity_copy, fl_gpu_colouring_copy, fl_gpu_make_global_numbering_p2, &
            fl_gpu_assemble_advdif_cg, fl_gpu_apply_dirichlet, fl_gpu_petsc_solve, &
            fl_gpu_pattern_register, fl_dev_petsc_solve, fl_amg_create, fl_amg_solve, fl_amg_destroy, &
            fl_batch_create, fl_batch_add, fl_batch_run, fl_batch_destroy, fl_set_assembly_tiles
  public :: fl_divergence_params, fl_gpu_secondorder_register, fl_dev_assemble_divergence_cg, &
            fl_dev_lumped_mass, fl_dev_mult_div_vector_div_T, fl_dev_mult_div_invscalar_div_T, &
            fl_dev_assemble_kmk, fl_dev_masslumped_poisson_rhs, fl_dev_correct_masslumped_velocity, &
            fl_dev_csr_addto
  public :: gpu_check

  integer(c_int), parameter, public :: FL_OK = 0

  type, bind(c) :: fl_mesh_desc
     integer(c_int32_t) :: nodes, elements, loc, index_base
     type(c_ptr) :: ndglno
     integer(c_int32_t) :: x_nodes
     type(c_ptr) :: x_ndglno
     type(c_ptr) :: coords
  end type fl_mesh_desc

  type, bind(c) :: fl_advdif_params
     real(c_double) :: theta, dt, beta
     integer(c_int32_t) :: have_mass, lump_mass, have_advection, have_diffusivity
     integer(c_int32_t) :: isotropic_diffusivity, have_source, have_absorption, quad_degree
     real(c_double) :: diffusivity(9)
  end type fl_advdif_params

  type, bind(c) :: fl_fields
     type(c_ptr) :: t, velocity, source, absorption
  end type fl_fields

  type, bind(c) :: fl_solver_opts
     integer(c_int32_t) :: ksp_type, restart
     real(c_double) :: rtol, atol, dtol
     integer(c_int32_t) :: max_its, start_from_zero, precision
     real(c_double) :: inner_rtol
  end type fl_solver_opts

  ! assemble_divergence_matrix_cg options and surface mesh (by parts)
  type, bind(c) :: fl_divergence_params
     integer(c_int32_t) :: integrate_by_parts, nfaces, index_base, pad
     type(c_ptr) :: faces, face_ele, bc_type, bc_val
  end type fl_divergence_params

  type, bind(c) :: fl_solve_report
     integer(c_int32_t) :: iterations, reason
     real(c_double) :: final_rnorm, rnorm0, true_rel_residual
     integer(c_int32_t) :: outer_iterations, pad
  end type fl_solve_report

  interface
     function fl_last_error() bind(c, name="fl_last_error") result(msg)
       import :: c_ptr
       type(c_ptr) :: msg
     end function fl_last_error

     function fl_gpu_mesh_register(desc, handle) bind(c, name="fl_gpu_mesh_register") result(st)
       import :: c_int, c_ptr, fl_mesh_desc
       type(fl_mesh_desc), intent(in) :: desc
       type(c_ptr), intent(out) :: handle
       integer(c_int) :: st
     end function fl_gpu_mesh_register

     function fl_gpu_mesh_destroy(handle) bind(c, name="fl_gpu_mesh_destroy") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: handle
       integer(c_int) :: st
     end function fl_gpu_mesh_destroy

     function fl_gpu_mesh_info(handle, nnz, ncolours) bind(c, name="fl_gpu_mesh_info") result(st)
       import :: c_int, c_ptr, c_int64_t, c_int32_t
       type(c_ptr), value :: handle
       integer(c_int64_t), intent(out) :: nnz
       integer(c_int32_t), intent(out) :: ncolours
       integer(c_int) :: st
     end function fl_gpu_mesh_info

     function fl_gpu_sparsity_copy(handle, findrm, colm, centrm, base) &
          bind(c, name="fl_gpu_sparsity_copy") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: handle, findrm, colm, centrm
       integer(c_int32_t), value :: base
       integer(c_int) :: st
     end function fl_gpu_sparsity_copy

     function fl_gpu_colouring_copy(handle, colour, colour_ptr, colour_elems, base) &
          bind(c, name="fl_gpu_colouring_copy") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: handle, colour, colour_ptr, colour_elems
       integer(c_int32_t), value :: base
       integer(c_int) :: st
     end function fl_gpu_colouring_copy

     function fl_gpu_make_global_numbering_p2(nvert, elements, ndglno_p1, base, ndglno_p2, n2) &
          bind(c, name="fl_gpu_make_global_numbering_p2") result(st)
       import :: c_int, c_ptr, c_int32_t
       integer(c_int32_t), value :: nvert, elements, base
       type(c_ptr), value :: ndglno_p1, ndglno_p2
       integer(c_int32_t), intent(out) :: n2
       integer(c_int) :: st
     end function fl_gpu_make_global_numbering_p2

     function fl_gpu_assemble_advdif_cg(handle, params, fields, val, rhs) &
          bind(c, name="fl_gpu_assemble_advdif_cg") result(st)
       import :: c_int, c_ptr, fl_advdif_params, fl_fields
       type(c_ptr), value :: handle
       type(fl_advdif_params), intent(in) :: params
       type(fl_fields), intent(in) :: fields
       type(c_ptr), value :: val, rhs
       integer(c_int) :: st
     end function fl_gpu_assemble_advdif_cg

     function fl_gpu_apply_dirichlet(handle, nb, nodes, base, g, t, dt, rhs, inactive) &
          bind(c, name="fl_gpu_apply_dirichlet") result(st)
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: handle, nodes, g, t, rhs, inactive
       integer(c_int32_t), value :: nb, base
       real(c_double), value :: dt
       integer(c_int) :: st
     end function fl_gpu_apply_dirichlet

     function fl_gpu_petsc_solve(handle, opts, val, inactive, rhs, x, report) &
          bind(c, name="fl_gpu_petsc_solve") result(st)
       import :: c_int, c_ptr, fl_solver_opts, fl_solve_report
       type(c_ptr), value :: handle
       type(fl_solver_opts), intent(in) :: opts
       type(c_ptr), value :: val, inactive, rhs, x
       type(fl_solve_report), intent(out) :: report
       integer(c_int) :: st
     end function fl_gpu_petsc_solve

     ! device-pointer solve (arrays already on the GPU, e.g. from
     ! fl_dev_assemble_advdif_cg); stream may be c_null_ptr
     function fl_dev_petsc_solve(handle, opts, val, inactive, rhs, x, report, stream) &
          bind(c, name="fl_dev_petsc_solve") result(st)
       import :: c_int, c_ptr, fl_solver_opts, fl_solve_report
       type(c_ptr), value :: handle
       type(fl_solver_opts), intent(in) :: opts
       type(c_ptr), value :: val, inactive, rhs, x, stream
       type(fl_solve_report), intent(out) :: report
       integer(c_int) :: st
     end function fl_dev_petsc_solve

     ! a handle for a matrix read from a matrixdump (tools/petsc_readnsolve.F90)
     function fl_gpu_pattern_register(n, findrm, colm, base, handle) &
          bind(c, name="fl_gpu_pattern_register") result(st)
       import :: c_int, c_ptr, c_int32_t
       integer(c_int32_t), value :: n, base
       type(c_ptr), value :: findrm, colm
       type(c_ptr), intent(out) :: handle
       integer(c_int) :: st
     end function fl_gpu_pattern_register

     ! smoothed-aggregation AMG for CG (the gamg preconditioner option);
     ! device pointers, the hierarchy is reused while the matrix is unchanged
     ! (cache_solver_context)
     function fl_amg_create(handle, val, inactive, stream, amg) bind(c, name="fl_amg_create") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: handle, val, inactive, stream
       type(c_ptr), intent(out) :: amg
       integer(c_int) :: st
     end function fl_amg_create

     function fl_amg_solve(amg, opts, rhs, x, report, stream) bind(c, name="fl_amg_solve") result(st)
       import :: c_int, c_ptr, fl_solver_opts, fl_solve_report
       type(c_ptr), value :: amg, rhs, x, stream
       type(fl_solver_opts), intent(in) :: opts
       type(fl_solve_report), intent(out) :: report
       integer(c_int) :: st
     end function fl_amg_solve

     function fl_amg_destroy(amg) bind(c, name="fl_amg_destroy") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: amg
       integer(c_int) :: st
     end function fl_amg_destroy

     ! several solve_field_equation_cg steps (fields or meshes) as CUDA graphs
     function fl_batch_create(batch) bind(c, name="fl_batch_create") result(st)
       import :: c_int, c_ptr
       type(c_ptr), intent(out) :: batch
       integer(c_int) :: st
     end function fl_batch_create

     function fl_batch_add(batch, handle, params, fields, nb, bc_nodes, base, bc_values, opts, &
          val, rhs, inactive, x) bind(c, name="fl_batch_add") result(st)
       import :: c_int, c_ptr, c_int32_t, fl_advdif_params, fl_fields, fl_solver_opts
       type(c_ptr), value :: batch, handle, bc_nodes, bc_values, val, rhs, inactive, x
       type(fl_advdif_params), intent(in) :: params
       type(fl_fields), intent(in) :: fields
       type(fl_solver_opts), intent(in) :: opts
       integer(c_int32_t), value :: nb, base
       integer(c_int) :: st
     end function fl_batch_add

     function fl_batch_run(batch, stream, reports) bind(c, name="fl_batch_run") result(st)
       import :: c_int, c_ptr, fl_solve_report
       type(c_ptr), value :: batch, stream
       type(fl_solve_report), intent(out) :: reports(*)
       integer(c_int) :: st
     end function fl_batch_run

     function fl_batch_destroy(batch) bind(c, name="fl_batch_destroy") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: batch
       integer(c_int) :: st
     end function fl_batch_destroy

     function fl_set_assembly_tiles(handle, elem_block, elem_blocks_per_sm, row_tile) &
          bind(c, name="fl_set_assembly_tiles") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: handle
       integer(c_int32_t), value :: elem_block, elem_blocks_per_sm, row_tile
       integer(c_int) :: st
     end function fl_set_assembly_tiles

     ! pressure projection, P1 pressure and P1 velocity on one mesh
     ! (device pointers; block_csr_matrix blocks as c_loc of each block's val)
     function fl_gpu_secondorder_register(handle, out) bind(c, name="fl_gpu_secondorder_register") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: handle
       type(c_ptr), intent(out) :: out
       integer(c_int) :: st
     end function fl_gpu_secondorder_register

     function fl_dev_assemble_divergence_cg(handle, params, ct_val, ct_rhs, div_mass_lumped, &
          grad_mass_lumped, stream) bind(c, name="fl_dev_assemble_divergence_cg") result(st)
       import :: c_int, c_ptr, fl_divergence_params
       type(c_ptr), value :: handle, ct_rhs, div_mass_lumped, grad_mass_lumped, stream
       type(fl_divergence_params), intent(in) :: params
       type(c_ptr), intent(in) :: ct_val(3)
       integer(c_int) :: st
     end function fl_dev_assemble_divergence_cg

     function fl_dev_lumped_mass(handle, lumped_mass, stream) bind(c, name="fl_dev_lumped_mass") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: handle, lumped_mass, stream
       integer(c_int) :: st
     end function fl_dev_lumped_mass

     function fl_dev_mult_div_vector_div_T(product, ndim, a_val, w, b_val, out, stream) &
          bind(c, name="fl_dev_mult_div_vector_div_T") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: product, w, out, stream
       integer(c_int32_t), value :: ndim
       type(c_ptr), intent(in) :: a_val(3), b_val(3)
       integer(c_int) :: st
     end function fl_dev_mult_div_vector_div_T

     function fl_dev_mult_div_invscalar_div_T(product, a_val, s_val, b_val, out, stream) &
          bind(c, name="fl_dev_mult_div_invscalar_div_T") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: product, a_val, s_val, b_val, out, stream
       integer(c_int) :: st
     end function fl_dev_mult_div_invscalar_div_T

     function fl_dev_assemble_kmk(handle, product, theta_pg, p_masslump, kt_val, kmk_val, stream) &
          bind(c, name="fl_dev_assemble_kmk") result(st)
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: handle, product, p_masslump, kt_val, kmk_val, stream
       real(c_double), value :: theta_pg
       integer(c_int) :: st
     end function fl_dev_assemble_kmk

     function fl_dev_masslumped_poisson_rhs(handle, ctp_val, mom_rhs, ct_rhs, inverse_masslump, velocity, &
          dt, theta_pg, poisson_rhs, stream) bind(c, name="fl_dev_masslumped_poisson_rhs") result(st)
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: handle, mom_rhs, ct_rhs, inverse_masslump, velocity, poisson_rhs, stream
       type(c_ptr), intent(in) :: ctp_val(3)
       real(c_double), value :: dt, theta_pg
       integer(c_int) :: st
     end function fl_dev_masslumped_poisson_rhs

     function fl_dev_correct_masslumped_velocity(handle, ct_val, inverse_masslump, delta_p, velocity, stream) &
          bind(c, name="fl_dev_correct_masslumped_velocity") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: handle, inverse_masslump, delta_p, velocity, stream
       type(c_ptr), intent(in) :: ct_val(3)
       integer(c_int) :: st
     end function fl_dev_correct_masslumped_velocity

     function fl_dev_csr_addto(pattern, val, other, scale, stream) bind(c, name="fl_dev_csr_addto") result(st)
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: pattern, val, other, stream
       real(c_double), value :: scale
       integer(c_int) :: st
     end function fl_dev_csr_addto
  end interface

contains

  subroutine gpu_check(st, where)
    !!< FLAbort on a usage error returned by the library.
    integer(c_int), intent(in) :: st
    character(len=*), intent(in) :: where
    character(kind=c_char), pointer :: msg(:)
    character(len=1024) :: text
    integer :: i

    if (st == FL_OK) return
    call c_f_pointer(fl_last_error(), msg, (/ 1024 /))
    text = ""
    do i = 1, 1024
       if (msg(i) == c_null_char) exit
       text(i:i) = msg(i)
    end do
    ewrite(-1, *) trim(where), ": ", trim(text)
    FLAbort("GPU CG path failed")
  end subroutine gpu_check

end module fl_gpu_bindings
