!    fl_gpu_bindings.F90 -- ISO_C_BINDING interface to libfluidity_gb300.so.
!
!    The Fortran side of the drop-in boundary:
!
!    * bind(c) types and an explicit interface for every entry point declared
!      in include/fluidity_gb300.h (same names, same argument order);
!    * wrappers with the argument lists of the reference routines they stand
!      in for, taking Fluidity's own types (scalar_field, csr_matrix,
!      state_type) and passing c_loc() pointers to the arrays those types
!      already own:
!
!        gpu_assemble_advection_diffusion_cg(t, matrix, rhs, state, dt, velocity_name)
!            -> assemble_advection_diffusion_cg (assemble/Advection_Diffusion_CG.F90:228)
!        gpu_petsc_solve_scalar(x, matrix, rhs, option_path, iterations_taken)
!            -> petsc_solve_scalar (femtools/Solvers.F90:111)
!        gpu_solve_field_equation_cg(field_name, state, istate, dt, velocity_name, iterations_taken)
!            -> solve_field_equation_cg (assemble/Advection_Diffusion_CG.F90:127)
!
!      gpu_advdif_cg_supported(t, state) and gpu_petsc_solve_supported(option_path)
!      tell a caller whether the options in force are ones the GPU path
!      implements (otherwise the caller keeps the reference routine);
!    * a cache of mesh handles keyed like the reference's transform cache
!      (femtools/Transform_elements.F90:131-168): the coordinate field's
!      refcount%id, the field mesh's refcount%id and the mesh-movement event
!      count; a moved or adapted mesh is registered again.
!
!    Status handling follows the reference: usage errors abort with FLAbort
!    (include/fdebug.h:56); solver divergence is reported as in
!    ConvergenceCheck (femtools/Solvers.F90:1369-1479): a warning on stderr,
!    and sig_int set (dump and finish at the end of the step) unless the
!    solver options allow the failure.
!
!    Not compiled in this repository (no Fortran compiler is available): it is
!    compiled into Fluidity's femtools library next to the modules it uses.
#include "fdebug.h"
module fl_gpu_bindings
  use iso_c_binding
  use fldebug
  use global_parameters, only: FIELD_NAME_LEN, OPTION_PATH_LEN
  use spud
  use eventcounter, only: eventcount, EVENT_MESH_MOVEMENT
  use signal_vars, only: sig_int
  use elements
  use sparse_tools
  use fields
  use state_module
  use boundary_conditions
  use field_options, only: complete_field_path
  use sparsity_patterns_meshes, only: get_csr_sparsity_firstorder
  implicit none
  private

  public :: fl_mesh_desc, fl_advdif_params, fl_fields, fl_solver_opts, fl_solve_report, &
            fl_divergence_params, fl_face_bcs
  public :: fl_last_error, fl_gpu_mesh_register, fl_gpu_mesh_destroy, fl_gpu_pattern_register, &
            fl_gpu_mesh_info, fl_gpu_sparsity_copy, fl_gpu_colouring_copy, &
            fl_gpu_make_global_numbering_p2, fl_gpu_assemble_advdif_cg, fl_dev_assemble_advdif_cg, &
            fl_dev_assemble_advdif_faces, fl_gpu_assemble_advdif_faces, &
            fl_dev_assemble_p1_diffusion_noalloc, fl_gpu_apply_dirichlet, fl_dev_apply_dirichlet, &
            fl_gpu_petsc_solve, fl_dev_petsc_solve, fl_dev_solve_field_equation_cg, fl_dev_csr_mult, &
            fl_dev_autotune_assembly, &
            fl_set_assembly_tiles, fl_get_assembly_tiles, fl_batch_create, fl_batch_add, fl_batch_run, &
            fl_batch_size, fl_batch_destroy, fl_amg_create, fl_amg_solve, fl_amg_levels, &
            fl_amg_set_norm, fl_amg_set_precision, fl_amg_destroy, fl_gnn_num_params, fl_gnn_create, &
            fl_gnn_destroy, fl_gnn_set_weights, fl_gnn_set_loss, fl_gnn_get_weights, fl_gnn_predict, &
            fl_gnn_gradients, fl_gnn_train_step, fl_gpu_secondorder_register, &
            fl_dev_assemble_divergence_cg, fl_dev_lumped_mass, fl_dev_mult_div_vector_div_T, &
            fl_dev_mult_div_invscalar_div_T, fl_dev_assemble_kmk, fl_dev_masslumped_poisson_rhs, &
            fl_dev_correct_masslumped_velocity, fl_dev_csr_addto, fl_kernel_launch_count, &
            fl_set_kernel_timing, fl_last_assembly_kernel_ms, fl_set_wait_test, fl_dev_projected_guess, &
            fl_gpu_rect_register, fl_dev_assemble_divergence_p2p1, fl_dev_assemble_divergence_p2p1_faces, &
            fl_gpu_rect_secondorder_register
  public :: gpu_check, gpu_mesh_handle, gpu_advdif_cg_supported, gpu_assemble_advection_diffusion_cg, &
            gpu_petsc_solve_supported, gpu_petsc_solve_scalar, gpu_solve_field_equation_cg

  integer(c_int), parameter, public :: FL_OK = 0
  integer, parameter :: BC_TYPE_WEAKDIRICHLET = 2, BC_TYPE_INTERNAL = 3

  ! ---------------------------------------------------------------- types --
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
     integer(c_int32_t) :: integrate_advection_by_parts, pad
  end type fl_advdif_params

  type, bind(c) :: fl_fields
     type(c_ptr) :: t, velocity, source, absorption
  end type fl_fields

  type, bind(c) :: fl_face_bcs
     integer(c_int32_t) :: nfaces, floc, index_base, pad
     type(c_ptr) :: faces, xfaces, face_ele, bc_type, bc_value, bc_value2
  end type fl_face_bcs

  type, bind(c) :: fl_solver_opts
     integer(c_int32_t) :: ksp_type, restart
     real(c_double) :: rtol, atol, dtol
     integer(c_int32_t) :: max_its, start_from_zero, precision
     real(c_double) :: inner_rtol
     integer(c_int32_t) :: norm_type, schedule
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

  ! a registered mesh (or pattern) and the key it was registered under
  type gpu_mesh_entry
     integer :: x_id = -1, t_id = -1, movement = -1
     type(c_ptr) :: handle = c_null_ptr
  end type gpu_mesh_entry
  integer, parameter :: CACHE_SIZE = 16
  type(gpu_mesh_entry), dimension(CACHE_SIZE), save :: mesh_cache
  type(gpu_mesh_entry), dimension(CACHE_SIZE), save :: pattern_cache
  integer, save :: mesh_next = 1, pattern_next = 1

  ! ----------------------------------------------------------- interfaces --
  interface
     function fl_last_error() bind(c, name="fl_last_error") result(msg)
       import :: c_ptr
       type(c_ptr) :: msg
     end function fl_last_error

     function fl_gpu_mesh_register(desc, out) bind(c, name="fl_gpu_mesh_register") result(st)
       import :: c_int, c_ptr, fl_mesh_desc
       type(fl_mesh_desc), intent(in) :: desc
       type(c_ptr), intent(out) :: out
       integer(c_int) :: st
     end function fl_gpu_mesh_register

     function fl_gpu_mesh_destroy(mesh) bind(c, name="fl_gpu_mesh_destroy") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: mesh
       integer(c_int) :: st
     end function fl_gpu_mesh_destroy

     ! a handle for a matrix pattern alone (tools/petsc_readnsolve.F90, or a
     ! csr_matrix whose mesh is not registered)
     function fl_gpu_pattern_register(n, findrm, colm, index_base, out) &
          bind(c, name="fl_gpu_pattern_register") result(st)
       import :: c_int, c_ptr, c_int32_t
       integer(c_int32_t), value :: n, index_base
       type(c_ptr), value :: findrm, colm
       type(c_ptr), intent(out) :: out
       integer(c_int) :: st
     end function fl_gpu_pattern_register

     function fl_gpu_mesh_info(mesh, nnz, ncolours) bind(c, name="fl_gpu_mesh_info") result(st)
       import :: c_int, c_ptr, c_int64_t, c_int32_t
       type(c_ptr), value :: mesh
       integer(c_int64_t), intent(out) :: nnz
       integer(c_int32_t), intent(out) :: ncolours
       integer(c_int) :: st
     end function fl_gpu_mesh_info

     function fl_gpu_sparsity_copy(mesh, findrm, colm, centrm, index_base) &
          bind(c, name="fl_gpu_sparsity_copy") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: mesh, findrm, colm, centrm
       integer(c_int32_t), value :: index_base
       integer(c_int) :: st
     end function fl_gpu_sparsity_copy

     function fl_gpu_colouring_copy(mesh, colour, colour_ptr, colour_elems, index_base) &
          bind(c, name="fl_gpu_colouring_copy") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: mesh, colour, colour_ptr, colour_elems
       integer(c_int32_t), value :: index_base
       integer(c_int) :: st
     end function fl_gpu_colouring_copy

     function fl_gpu_make_global_numbering_p2(nvert, elements, ndglno_p1, index_base, ndglno_p2, n2) &
          bind(c, name="fl_gpu_make_global_numbering_p2") result(st)
       import :: c_int, c_ptr, c_int32_t
       integer(c_int32_t), value :: nvert, elements, index_base
       type(c_ptr), value :: ndglno_p1, ndglno_p2
       integer(c_int32_t), intent(out) :: n2
       integer(c_int) :: st
     end function fl_gpu_make_global_numbering_p2

     function fl_gpu_assemble_advdif_cg(mesh, params, fields, val, rhs) &
          bind(c, name="fl_gpu_assemble_advdif_cg") result(st)
       import :: c_int, c_ptr, fl_advdif_params, fl_fields
       type(c_ptr), value :: mesh
       type(fl_advdif_params), intent(in) :: params
       type(fl_fields), intent(in) :: fields
       type(c_ptr), value :: val, rhs
       integer(c_int) :: st
     end function fl_gpu_assemble_advdif_cg

     function fl_dev_assemble_advdif_cg(mesh, params, fields, val, rhs, stream) &
          bind(c, name="fl_dev_assemble_advdif_cg") result(st)
       import :: c_int, c_ptr, fl_advdif_params, fl_fields
       type(c_ptr), value :: mesh
       type(fl_advdif_params), intent(in) :: params
       type(fl_fields), intent(in) :: fields
       type(c_ptr), value :: val, rhs, stream
       integer(c_int) :: st
     end function fl_dev_assemble_advdif_cg

     function fl_dev_assemble_advdif_faces(mesh, params, faces, fields, val, rhs, stream) &
          bind(c, name="fl_dev_assemble_advdif_faces") result(st)
       import :: c_int, c_ptr, fl_advdif_params, fl_face_bcs, fl_fields
       type(c_ptr), value :: mesh
       type(fl_advdif_params), intent(in) :: params
       type(fl_face_bcs), intent(in) :: faces
       type(fl_fields), intent(in) :: fields
       type(c_ptr), value :: val, rhs, stream
       integer(c_int) :: st
     end function fl_dev_assemble_advdif_faces

     function fl_gpu_assemble_advdif_faces(mesh, params, faces, fields, val, rhs) &
          bind(c, name="fl_gpu_assemble_advdif_faces") result(st)
       import :: c_int, c_ptr, fl_advdif_params, fl_face_bcs, fl_fields
       type(c_ptr), value :: mesh
       type(fl_advdif_params), intent(in) :: params
       type(fl_face_bcs), intent(in) :: faces
       type(fl_fields), intent(in) :: fields
       type(c_ptr), value :: val, rhs
       integer(c_int) :: st
     end function fl_gpu_assemble_advdif_faces

     function fl_dev_assemble_p1_diffusion_noalloc(mesh, params, fields, val, rhs, stream) &
          bind(c, name="fl_dev_assemble_p1_diffusion_noalloc") result(st)
       import :: c_int, c_ptr, fl_advdif_params, fl_fields
       type(c_ptr), value :: mesh
       type(fl_advdif_params), intent(in) :: params
       type(fl_fields), intent(in) :: fields
       type(c_ptr), value :: val, rhs, stream
       integer(c_int) :: st
     end function fl_dev_assemble_p1_diffusion_noalloc

     function fl_gpu_apply_dirichlet(mesh, nb, nodes, index_base, g, t, dt, rhs, inactive) &
          bind(c, name="fl_gpu_apply_dirichlet") result(st)
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: mesh, nodes, g, t, rhs, inactive
       integer(c_int32_t), value :: nb, index_base
       real(c_double), value :: dt
       integer(c_int) :: st
     end function fl_gpu_apply_dirichlet

     function fl_dev_apply_dirichlet(mesh, nb, nodes, index_base, g, t, dt, rhs, inactive, stream) &
          bind(c, name="fl_dev_apply_dirichlet") result(st)
       import :: c_int, c_ptr, c_int32_t, c_double
       type(c_ptr), value :: mesh, nodes, g, t, rhs, inactive, stream
       integer(c_int32_t), value :: nb, index_base
       real(c_double), value :: dt
       integer(c_int) :: st
     end function fl_dev_apply_dirichlet

     function fl_gpu_petsc_solve(mesh, opts, val, inactive, rhs, x, report) &
          bind(c, name="fl_gpu_petsc_solve") result(st)
       import :: c_int, c_ptr, fl_solver_opts, fl_solve_report
       type(c_ptr), value :: mesh
       type(fl_solver_opts), intent(in) :: opts
       type(c_ptr), value :: val, inactive, rhs, x
       type(fl_solve_report), intent(out) :: report
       integer(c_int) :: st
     end function fl_gpu_petsc_solve

     function fl_dev_petsc_solve(mesh, opts, val, inactive, rhs, x, report, stream) &
          bind(c, name="fl_dev_petsc_solve") result(st)
       import :: c_int, c_ptr, fl_solver_opts, fl_solve_report
       type(c_ptr), value :: mesh
       type(fl_solver_opts), intent(in) :: opts
       type(c_ptr), value :: val, inactive, rhs, x, stream
       type(fl_solve_report), intent(out) :: report
       integer(c_int) :: st
     end function fl_dev_petsc_solve

     function fl_dev_solve_field_equation_cg(mesh, params, fields, nb, bc_nodes, index_base, bc_values, &
          opts, val, rhs, inactive, delta, t_new, report, stream) &
          bind(c, name="fl_dev_solve_field_equation_cg") result(st)
       import :: c_int, c_ptr, c_int32_t, fl_advdif_params, fl_fields, fl_solver_opts, fl_solve_report
       type(c_ptr), value :: mesh
       type(fl_advdif_params), intent(in) :: params
       type(fl_fields), intent(in) :: fields
       integer(c_int32_t), value :: nb, index_base
       type(c_ptr), value :: bc_nodes, bc_values
       type(fl_solver_opts), intent(in) :: opts
       type(c_ptr), value :: val, rhs, inactive, delta, t_new
       type(fl_solve_report), intent(out) :: report
       type(c_ptr), value :: stream
       integer(c_int) :: st
     end function fl_dev_solve_field_equation_cg

     function fl_dev_csr_mult(mesh, val, x, y, stream) bind(c, name="fl_dev_csr_mult") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: mesh, val, x, y, stream
       integer(c_int) :: st
     end function fl_dev_csr_mult

     function fl_dev_autotune_assembly(mesh, params, fields, val, rhs, stream, tiles) &
          bind(c, name="fl_dev_autotune_assembly") result(st)
       import :: c_int, c_ptr, c_int32_t, fl_advdif_params, fl_fields
       type(c_ptr), value :: mesh, val, rhs, stream
       type(fl_advdif_params), intent(in) :: params
       type(fl_fields), intent(in) :: fields
       integer(c_int32_t), intent(out) :: tiles(3)
       integer(c_int) :: st
     end function fl_dev_autotune_assembly

     function fl_set_assembly_tiles(mesh, elem_block, elem_blocks_per_sm, row_tile) &
          bind(c, name="fl_set_assembly_tiles") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: mesh
       integer(c_int32_t), value :: elem_block, elem_blocks_per_sm, row_tile
       integer(c_int) :: st
     end function fl_set_assembly_tiles

     function fl_get_assembly_tiles(mesh, tiles) bind(c, name="fl_get_assembly_tiles") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: mesh
       integer(c_int32_t), intent(out) :: tiles(3)
       integer(c_int) :: st
     end function fl_get_assembly_tiles

     ! several solve_field_equation_cg steps (fields or meshes) as CUDA graphs
     function fl_batch_create(batch) bind(c, name="fl_batch_create") result(st)
       import :: c_int, c_ptr
       type(c_ptr), intent(out) :: batch
       integer(c_int) :: st
     end function fl_batch_create

     function fl_batch_add(batch, mesh, params, fields, nb, bc_nodes, index_base, bc_values, opts, &
          val, rhs, inactive, x) bind(c, name="fl_batch_add") result(st)
       import :: c_int, c_ptr, c_int32_t, fl_advdif_params, fl_fields, fl_solver_opts
       type(c_ptr), value :: batch, mesh, bc_nodes, bc_values, val, rhs, inactive, x
       type(fl_advdif_params), intent(in) :: params
       type(fl_fields), intent(in) :: fields
       type(fl_solver_opts), intent(in) :: opts
       integer(c_int32_t), value :: nb, index_base
       integer(c_int) :: st
     end function fl_batch_add

     function fl_batch_run(batch, stream, reports) bind(c, name="fl_batch_run") result(st)
       import :: c_int, c_ptr, fl_solve_report
       type(c_ptr), value :: batch, stream
       type(fl_solve_report), intent(out) :: reports(*)
       integer(c_int) :: st
     end function fl_batch_run

     function fl_batch_size(batch) bind(c, name="fl_batch_size") result(n)
       import :: c_int, c_ptr
       type(c_ptr), value :: batch
       integer(c_int) :: n
     end function fl_batch_size

     function fl_batch_destroy(batch) bind(c, name="fl_batch_destroy") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: batch
       integer(c_int) :: st
     end function fl_batch_destroy

     ! smoothed-aggregation AMG for CG (the gamg preconditioner option);
     ! device pointers, the hierarchy is reused while the matrix is unchanged
     ! (cache_solver_context)
     function fl_amg_create(mesh, val, inactive, stream, amg) bind(c, name="fl_amg_create") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: mesh, val, inactive, stream
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

     function fl_amg_levels(amg, levels, rows, nnz, capacity) bind(c, name="fl_amg_levels") result(st)
       import :: c_int, c_ptr, c_int32_t, c_int64_t
       type(c_ptr), value :: amg
       integer(c_int32_t), intent(out) :: levels
       integer(c_int64_t), intent(out) :: rows(*), nnz(*)
       integer(c_int32_t), value :: capacity
       integer(c_int) :: st
     end function fl_amg_levels

     function fl_amg_set_norm(amg, unpreconditioned) bind(c, name="fl_amg_set_norm") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: amg
       integer(c_int32_t), value :: unpreconditioned
       integer(c_int) :: st
     end function fl_amg_set_norm

     function fl_amg_set_precision(amg, fp32) bind(c, name="fl_amg_set_precision") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: amg
       integer(c_int32_t), value :: fp32
       integer(c_int) :: st
     end function fl_amg_set_precision

     function fl_amg_destroy(amg) bind(c, name="fl_amg_destroy") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: amg
       integer(c_int) :: st
     end function fl_amg_destroy

     ! learned warm start of the pressure solve (device pointers)
     function fl_gnn_num_params() bind(c, name="fl_gnn_num_params") result(n)
       import :: c_int
       integer(c_int) :: n
     end function fl_gnn_num_params

     function fl_gnn_create(mesh, net) bind(c, name="fl_gnn_create") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: mesh
       type(c_ptr), intent(out) :: net
       integer(c_int) :: st
     end function fl_gnn_create

     function fl_gnn_destroy(net) bind(c, name="fl_gnn_destroy") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: net
       integer(c_int) :: st
     end function fl_gnn_destroy

     function fl_gnn_set_weights(net, weights, count) bind(c, name="fl_gnn_set_weights") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: net, weights
       integer(c_int32_t), value :: count
       integer(c_int) :: st
     end function fl_gnn_set_weights

     function fl_gnn_set_loss(net, val) bind(c, name="fl_gnn_set_loss") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: net, val
       integer(c_int) :: st
     end function fl_gnn_set_loss

     function fl_gnn_get_weights(net, weights, count) bind(c, name="fl_gnn_get_weights") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: net, weights
       integer(c_int32_t), value :: count
       integer(c_int) :: st
     end function fl_gnn_get_weights

     function fl_gnn_predict(net, p1, p2, b, pred, stream) bind(c, name="fl_gnn_predict") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: net, p1, p2, b, pred, stream
       integer(c_int) :: st
     end function fl_gnn_predict

     function fl_gnn_gradients(net, p1, p2, b, target, mask, nact, grad, loss, stream) &
          bind(c, name="fl_gnn_gradients") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: net, p1, p2, b, target, mask, grad, loss, stream
       integer(c_int32_t), value :: nact
       integer(c_int) :: st
     end function fl_gnn_gradients

     function fl_gnn_train_step(net, p1, p2, b, target, mask, nact, lr, loss_dev, stream) &
          bind(c, name="fl_gnn_train_step") result(st)
       import :: c_int, c_ptr, c_int32_t, c_float
       type(c_ptr), value :: net, p1, p2, b, target, mask, loss_dev, stream
       integer(c_int32_t), value :: nact
       real(c_float), value :: lr
       integer(c_int) :: st
     end function fl_gnn_train_step

     ! pressure projection, P1 pressure and P1 velocity on one mesh
     ! (device pointers; block_csr_matrix blocks as c_loc of each block's val)
     function fl_gpu_secondorder_register(mesh, out) bind(c, name="fl_gpu_secondorder_register") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: mesh
       type(c_ptr), intent(out) :: out
       integer(c_int) :: st
     end function fl_gpu_secondorder_register

     function fl_dev_assemble_divergence_cg(mesh, params, ct_val, ct_rhs, div_mass_lumped, &
          grad_mass_lumped, stream) bind(c, name="fl_dev_assemble_divergence_cg") result(st)
       import :: c_int, c_ptr, fl_divergence_params
       type(c_ptr), value :: mesh, ct_rhs, div_mass_lumped, grad_mass_lumped, stream
       type(fl_divergence_params), intent(in) :: params
       type(c_ptr), intent(in) :: ct_val(3)
       integer(c_int) :: st
     end function fl_dev_assemble_divergence_cg

     ! Taylor-Hood pair: P2 velocity (the mesh), P1 pressure on its vertices
     function fl_gpu_rect_register(mesh, out) bind(c, name="fl_gpu_rect_register") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: mesh
       type(c_ptr), intent(out) :: out
       integer(c_int) :: st
     end function fl_gpu_rect_register

     function fl_dev_assemble_divergence_p2p1(mesh, pattern, integrate_by_parts, quad_degree, ct_val, stream) &
          bind(c, name="fl_dev_assemble_divergence_p2p1") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: mesh, pattern, stream
       integer(c_int32_t), value :: integrate_by_parts, quad_degree
       type(c_ptr), intent(in) :: ct_val(3)
       integer(c_int) :: st
     end function fl_dev_assemble_divergence_p2p1

     ! its by-parts surface loop: params%faces = pressure (vertex) face nodes,
     ! vfaces(6, nfaces) = the velocity face nodes, bc_val(3, 6, nfaces)
     function fl_dev_assemble_divergence_p2p1_faces(mesh, pattern, params, vfaces, quad_degree, ct_val, &
          ct_rhs, stream) bind(c, name="fl_dev_assemble_divergence_p2p1_faces") result(st)
       import :: c_int, c_ptr, c_int32_t, fl_divergence_params
       type(c_ptr), value :: mesh, pattern, vfaces, ct_rhs, stream
       type(fl_divergence_params), intent(in) :: params
       integer(c_int32_t), value :: quad_degree
       type(c_ptr), intent(in) :: ct_val(3)
       integer(c_int) :: st
     end function fl_dev_assemble_divergence_p2p1_faces

     ! the pattern of its cmc_m (C C^T through the velocity nodes)
     function fl_gpu_rect_secondorder_register(pattern, out) bind(c, name="fl_gpu_rect_secondorder_register") &
          result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: pattern
       type(c_ptr), intent(out) :: out
       integer(c_int) :: st
     end function fl_gpu_rect_secondorder_register

     function fl_dev_lumped_mass(mesh, lumped_mass, stream) bind(c, name="fl_dev_lumped_mass") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: mesh, lumped_mass, stream
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

     function fl_dev_assemble_kmk(mesh, product, theta_pg, p_masslump, kt_val, kmk_val, stream) &
          bind(c, name="fl_dev_assemble_kmk") result(st)
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: mesh, product, p_masslump, kt_val, kmk_val, stream
       real(c_double), value :: theta_pg
       integer(c_int) :: st
     end function fl_dev_assemble_kmk

     function fl_dev_masslumped_poisson_rhs(mesh, ctp_val, mom_rhs, ct_rhs, inverse_masslump, velocity, &
          dt, theta_pg, poisson_rhs, stream) bind(c, name="fl_dev_masslumped_poisson_rhs") result(st)
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: mesh, mom_rhs, ct_rhs, inverse_masslump, velocity, poisson_rhs, stream
       type(c_ptr), intent(in) :: ctp_val(3)
       real(c_double), value :: dt, theta_pg
       integer(c_int) :: st
     end function fl_dev_masslumped_poisson_rhs

     function fl_dev_correct_masslumped_velocity(mesh, ct_val, inverse_masslump, delta_p, velocity, stream) &
          bind(c, name="fl_dev_correct_masslumped_velocity") result(st)
       import :: c_int, c_ptr
       type(c_ptr), value :: mesh, inverse_masslump, delta_p, velocity, stream
       type(c_ptr), intent(in) :: ct_val(3)
       integer(c_int) :: st
     end function fl_dev_correct_masslumped_velocity

     function fl_dev_csr_addto(pattern, val, other, scale, stream) bind(c, name="fl_dev_csr_addto") result(st)
       import :: c_int, c_ptr, c_double
       type(c_ptr), value :: pattern, val, other, stream
       real(c_double), value :: scale
       integer(c_int) :: st
     end function fl_dev_csr_addto

     function fl_kernel_launch_count() bind(c, name="fl_kernel_launch_count") result(n)
       import :: c_long_long
       integer(c_long_long) :: n
     end function fl_kernel_launch_count

     function fl_set_kernel_timing(mesh, on) bind(c, name="fl_set_kernel_timing") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: mesh
       integer(c_int32_t), value :: on
       integer(c_int) :: st
     end function fl_set_kernel_timing

     function fl_last_assembly_kernel_ms(mesh, ms) bind(c, name="fl_last_assembly_kernel_ms") result(st)
       import :: c_int, c_ptr, c_float
       type(c_ptr), value :: mesh
       real(c_float), intent(out) :: ms
       integer(c_int) :: st
     end function fl_last_assembly_kernel_ms

     ! projected initial guess from earlier solutions (device pointers;
     ! basis is an array of k device addresses)
     function fl_dev_projected_guess(mesh, val, inactive, rhs, k, basis, x0, coef, stream) &
          bind(c, name="fl_dev_projected_guess") result(st)
       import :: c_int, c_ptr, c_int32_t
       type(c_ptr), value :: mesh, val, inactive, rhs, x0, coef, stream
       integer(c_int32_t), value :: k
       type(c_ptr), intent(in) :: basis(*)
       integer(c_int) :: st
     end function fl_dev_projected_guess

     ! failure injection for tests of the bounded device waits
     function fl_set_wait_test(withhold, wait_ms) bind(c, name="fl_set_wait_test") result(st)
       import :: c_int, c_int32_t, c_double
       integer(c_int32_t), value :: withhold
       real(c_double), value :: wait_ms
       integer(c_int) :: st
     end function fl_set_wait_test
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

  function gpu_mesh_handle(t, positions) result(handle)
    !!< The registered GPU mesh of field t with coordinates positions,
    !!< registered on first use and again whenever the coordinate field or
    !!< the field mesh is a new one (adaptivity) or the mesh has moved
    !!< (the keys of the reference's transform cache).
    type(scalar_field), intent(in), target :: t
    type(vector_field), intent(in), target :: positions
    type(c_ptr) :: handle

    type(fl_mesh_desc) :: desc
    integer :: i, movement
    integer(c_int32_t), dimension(:), pointer :: tnd, xnd

    movement = eventcount(EVENT_MESH_MOVEMENT)
    do i = 1, CACHE_SIZE
       if (mesh_cache(i)%x_id == positions%refcount%id .and. &
           mesh_cache(i)%t_id == t%mesh%refcount%id .and. &
           mesh_cache(i)%movement == movement .and. c_associated(mesh_cache(i)%handle)) then
          handle = mesh_cache(i)%handle
          return
       end if
    end do

    ! ndglno arrays are 1-based, element-major (loc entries per element)
    tnd => t%mesh%ndglno
    xnd => positions%mesh%ndglno
    desc%nodes = node_count(t)
    desc%elements = ele_count(t)
    desc%loc = ele_loc(t, 1)
    desc%index_base = 1
    desc%ndglno = c_loc(tnd(1))
    desc%x_nodes = node_count(positions)
    desc%x_ndglno = c_loc(xnd(1))
    ! positions%val(3, N): xyz per node, the layout the C-ABI expects
    desc%coords = c_loc(positions%val(1, 1))

    i = mesh_next
    if (c_associated(mesh_cache(i)%handle)) call gpu_check(fl_gpu_mesh_destroy(mesh_cache(i)%handle), &
         "fl_gpu_mesh_destroy")
    call gpu_check(fl_gpu_mesh_register(desc, mesh_cache(i)%handle), "fl_gpu_mesh_register")
    mesh_cache(i)%x_id = positions%refcount%id
    mesh_cache(i)%t_id = t%mesh%refcount%id
    mesh_cache(i)%movement = movement
    mesh_next = mod(mesh_next, CACHE_SIZE) + 1
    handle = mesh_cache(i)%handle
  end function gpu_mesh_handle

  function gpu_pattern_handle(matrix) result(handle)
    !!< A pattern-only handle for the sparsity of matrix (cached by the
    !!< sparsity's refcount%id).
    type(csr_matrix), intent(in), target :: matrix
    type(c_ptr) :: handle
    integer :: i

    do i = 1, CACHE_SIZE
       if (pattern_cache(i)%t_id == matrix%sparsity%refcount%id .and. c_associated(pattern_cache(i)%handle)) then
          handle = pattern_cache(i)%handle
          return
       end if
    end do
    i = pattern_next
    if (c_associated(pattern_cache(i)%handle)) call gpu_check(fl_gpu_mesh_destroy(pattern_cache(i)%handle), &
         "fl_gpu_mesh_destroy")
    call gpu_check(fl_gpu_pattern_register(int(size(matrix, 1), c_int32_t), c_loc(matrix%sparsity%findrm(1)), &
         c_loc(matrix%sparsity%colm(1)), 1_c_int32_t, pattern_cache(i)%handle), "fl_gpu_pattern_register")
    pattern_cache(i)%t_id = matrix%sparsity%refcount%id
    pattern_next = mod(pattern_next, CACHE_SIZE) + 1
    handle = pattern_cache(i)%handle
  end function gpu_pattern_handle

  logical function gpu_advdif_cg_supported(t, state, velocity_name) result(ok)
    !!< Whether the options of field t are ones the GPU element loop
    !!< implements: P1 or P2 field on P1 simplex coordinates, constant
    !!< diffusivity tensor, no stabilisation, no moving mesh, no sinking
    !!< velocity, no multiphase or compressible equation terms, velocity on
    !!< the coordinate mesh.  Otherwise the caller keeps
    !!< assemble_advection_diffusion_cg.
    type(scalar_field), intent(in) :: t
    type(state_type), intent(in) :: state
    character(len=*), optional, intent(in) :: velocity_name

    character(len=FIELD_NAME_LEN) :: lvelocity_name, eqn
    character(len=OPTION_PATH_LEN) :: cg
    type(vector_field), pointer :: positions, velocity
    type(tensor_field), pointer :: diffusivity
    type(scalar_field), pointer :: source
    integer :: stat

    ok = .false.
    cg = trim(t%option_path) // "/prognostic/spatial_discretisation/continuous_galerkin"
    if (t%mesh%continuity /= 0) return
    if (.not. (ele_loc(t, 1) == 4 .or. ele_loc(t, 1) == 10)) return
    positions => extract_vector_field(state, "Coordinate")
    if (positions%dim /= 3 .or. ele_loc(positions, 1) /= 4) return
    if (have_option(trim(cg) // "/stabilisation/streamline_upwind") .or. &
        have_option(trim(cg) // "/stabilisation/streamline_upwind_petrov_galerkin")) return
    if (have_option(trim(cg) // "/advection_terms/only_sinking_velocity")) return
    if (have_option("/mesh_adaptivity/mesh_movement")) return
    if (option_count("/material_phase/vector_field::Velocity/prognostic") > 1) return
    call get_option(trim(t%option_path) // "/prognostic/equation[0]/name", eqn, default="AdvectionDiffusion")
    if (trim(eqn) /= "AdvectionDiffusion") return
    source => extract_scalar_field(state, trim(t%name) // "SinkingVelocity", stat=stat)
    if (stat == 0) return
    source => extract_scalar_field(state, trim(t%name) // "Source", stat=stat)
    if (stat == 0) then
       if (have_option(trim(source%option_path) // "/diagnostic/add_directly_to_rhs")) return
    end if
    diffusivity => extract_tensor_field(state, trim(t%name) // "Diffusivity", stat=stat)
    if (stat == 0) then
       if (diffusivity%field_type /= FIELD_TYPE_CONSTANT) return
    end if
    lvelocity_name = "NonlinearVelocity"
    if (present(velocity_name)) lvelocity_name = velocity_name
    velocity => extract_vector_field(state, lvelocity_name, stat=stat)
    if (stat == 0) then
       if (.not. (velocity%mesh == positions%mesh)) return
    end if
    ok = .true.
  end function gpu_advdif_cg_supported

  subroutine gpu_assemble_advection_diffusion_cg(t, matrix, rhs, state, dt, velocity_name)
    !!< assemble_advection_diffusion_cg (Advection_Diffusion_CG.F90:228) on
    !!< the GPU, with the reference's argument list: the options are read as
    !!< the reference reads them (:384-465), the element loop and the surface
    !!< loop run on the device, and the strong Dirichlet conditions are
    !!< applied by the reference's own apply_dirichlet_conditions.
    !!< matrix%val and rhs%val receive the assembled system.
    type(scalar_field), intent(inout), target :: t
    type(csr_matrix), intent(inout), target :: matrix
    type(scalar_field), intent(inout), target :: rhs
    type(state_type), intent(inout) :: state
    real, intent(in) :: dt
    character(len=*), optional, intent(in) :: velocity_name

    character(len=FIELD_NAME_LEN) :: lvelocity_name
    character(len=OPTION_PATH_LEN) :: cg
    type(fl_advdif_params) :: params
    type(fl_fields) :: flds
    type(fl_face_bcs) :: fbcs
    type(c_ptr) :: handle
    type(vector_field), pointer :: positions, velocity
    type(scalar_field), pointer :: source, absorption
    type(tensor_field), pointer :: diffusivity
    type(scalar_field) :: t_bc, t_bc_2
    integer, dimension(:), allocatable :: t_bc_types
    integer(c_int32_t), dimension(:,:), allocatable, target :: faces, xfaces
    integer(c_int32_t), dimension(:), allocatable, target :: face_eles, bc_types
    real(c_double), dimension(:,:), allocatable, target :: bc1, bc2
    real :: theta, beta
    integer :: stat, i, a, b, nf, floc

    if (.not. gpu_advdif_cg_supported(t, state, velocity_name)) then
       FLAbort("gpu_assemble_advection_diffusion_cg: options not supported on the GPU path")
    end if
    cg = trim(t%option_path) // "/prognostic/spatial_discretisation/continuous_galerkin"
    positions => extract_vector_field(state, "Coordinate")
    handle = gpu_mesh_handle(t, positions)

    call get_option(trim(t%option_path) // "/prognostic/temporal_discretisation/theta", theta)
    call get_option(trim(t%option_path) // "/prognostic/spatial_discretisation/conservative_advection", beta)
    params%theta = theta
    params%dt = dt
    params%beta = beta
    params%have_advection = merge(0, 1, have_option(trim(cg) // "/advection_terms/exclude_advection_terms"))
    params%integrate_advection_by_parts = 0
    if (params%have_advection == 1 .and. &
        have_option(trim(cg) // "/advection_terms/integrate_advection_by_parts")) &
        params%integrate_advection_by_parts = 1
    params%have_mass = merge(0, 1, have_option(trim(cg) // "/mass_terms/exclude_mass_terms"))
    params%lump_mass = 0
    if (params%have_mass == 1 .and. have_option(trim(cg) // "/mass_terms/lump_mass_matrix")) params%lump_mass = 1
    params%quad_degree = t%mesh%shape%quadrature%degree
    params%pad = 0

    flds%t = c_loc(t%val(1))
    flds%velocity = c_null_ptr
    flds%source = c_null_ptr
    flds%absorption = c_null_ptr
    lvelocity_name = "NonlinearVelocity"
    if (present(velocity_name)) lvelocity_name = velocity_name
    velocity => extract_vector_field(state, lvelocity_name, stat=stat)
    if (stat == 0) then
       flds%velocity = c_loc(velocity%val(1, 1))
    else
       params%have_advection = 0   ! no velocity: the reference advects with zero
       params%integrate_advection_by_parts = 0
    end if
    source => extract_scalar_field(state, trim(t%name) // "Source", stat=stat)
    params%have_source = merge(1, 0, stat == 0)
    if (stat == 0) flds%source = c_loc(source%val(1))
    absorption => extract_scalar_field(state, trim(t%name) // "Absorption", stat=stat)
    params%have_absorption = merge(1, 0, stat == 0)
    if (stat == 0) flds%absorption = c_loc(absorption%val(1))
    diffusivity => extract_tensor_field(state, trim(t%name) // "Diffusivity", stat=stat)
    params%have_diffusivity = merge(1, 0, stat == 0)
    params%isotropic_diffusivity = 0
    params%diffusivity = 0.0
    if (stat == 0) then
       ! constant tensor field: one (dim, dim) value, row-major in the C-ABI
       do a = 1, 3
          do b = 1, 3
             params%diffusivity(3 * (a - 1) + b) = diffusivity%val(a, b, 1)
          end do
       end do
       if (option_count(complete_field_path(diffusivity%option_path)) == &
           option_count(trim(complete_field_path(diffusivity%option_path)) // "/value/isotropic")) &
           params%isotropic_diffusivity = 1
    end if

    ! element loop: zero(matrix), zero(rhs), coloured assembly, addto
    call gpu_check(fl_gpu_assemble_advdif_cg(handle, params, flds, c_loc(matrix%val(1)), c_loc(rhs%val(1))), &
         "fl_gpu_assemble_advdif_cg")

    ! surface loop (:608-640)
    if ((params%have_advection == 1 .and. params%integrate_advection_by_parts == 1) .or. &
        params%have_diffusivity == 1) then
       nf = surface_element_count(t)
       allocate(t_bc_types(nf))
       call get_entire_boundary_condition(t, &
            (/ "neumann      ", "weakdirichlet", "internal     ", "robin        " /), &
            t_bc, t_bc_types, boundary_second_value=t_bc_2)
       floc = face_loc(t, 1)
       allocate(faces(floc, nf), xfaces(3, nf), face_eles(nf), bc_types(nf), bc1(floc, nf), bc2(floc, nf))
       do i = 1, nf
          faces(:, i) = face_global_nodes(t, i)
          xfaces(:, i) = face_global_nodes(positions, i)
          face_eles(i) = face_ele(t, i)
          bc_types(i) = t_bc_types(i)
          bc1(:, i) = ele_val(t_bc, i)
          bc2(:, i) = ele_val(t_bc_2, i)
       end do
       fbcs%nfaces = nf
       fbcs%floc = floc
       fbcs%index_base = 1
       fbcs%pad = 0
       if (nf > 0) then
          fbcs%faces = c_loc(faces(1, 1))
          fbcs%xfaces = c_loc(xfaces(1, 1))
          fbcs%face_ele = c_loc(face_eles(1))
          fbcs%bc_type = c_loc(bc_types(1))
          fbcs%bc_value = c_loc(bc1(1, 1))
          fbcs%bc_value2 = c_loc(bc2(1, 1))
       else
          fbcs%faces = c_null_ptr
          fbcs%xfaces = c_null_ptr
          fbcs%face_ele = c_null_ptr
          fbcs%bc_type = c_null_ptr
          fbcs%bc_value = c_null_ptr
          fbcs%bc_value2 = c_null_ptr
       end if
       if (any(t_bc_types == BC_TYPE_WEAKDIRICHLET) .and. params%have_diffusivity == 1) then
          FLExit("Weak Dirichlet boundary conditions with diffusivity are not supported by CG advection-diffusion")
       end if
       call gpu_check(fl_gpu_assemble_advdif_faces(handle, params, fbcs, flds, c_loc(matrix%val(1)), &
            c_loc(rhs%val(1))), "fl_gpu_assemble_advdif_faces")
       call deallocate(t_bc)
       call deallocate(t_bc_2)
       deallocate(t_bc_types, faces, xfaces, face_eles, bc_types, bc1, bc2)
    end if

    ! strong Dirichlet conditions: the reference's own routine on the host
    call apply_dirichlet_conditions(matrix, rhs, t, dt)
  end subroutine gpu_assemble_advection_diffusion_cg

  function solver_path(option_path) result(path)
    !!< complete_solver_option_path (femtools/Solvers.F90:608-627)
    character(len=*), intent(in) :: option_path
    character(len=OPTION_PATH_LEN) :: path
    if (have_option(trim(option_path) // '/prognostic/solver')) then
       path = trim(option_path) // '/prognostic/solver'
    else if (have_option(trim(option_path) // '/diagnostic/solver')) then
       path = trim(option_path) // '/diagnostic/solver'
    else if (have_option(trim(option_path) // '/solver')) then
       path = trim(option_path) // '/solver'
    else
       ewrite(-1, *) 'option_path: ', trim(option_path)
       FLAbort("Missing solver element in provided option_path.")
    end if
  end function solver_path

  logical function gpu_petsc_solve_supported(option_path) result(ok)
    !!< Whether the solver options at option_path are ones the GPU solve
    !!< implements: cg or gmres with the jacobi or gamg preconditioner.
    character(len=*), intent(in) :: option_path
    character(len=OPTION_PATH_LEN) :: path
    character(len=FIELD_NAME_LEN) :: ksptype, pctype

    path = solver_path(option_path)
    call get_option(trim(path) // '/iterative_method[0]/name', ksptype)
    call get_option(trim(path) // '/preconditioner[0]/name', pctype)
    ok = (trim(ksptype) == 'cg' .or. trim(ksptype) == 'gmres') .and. &
         (trim(pctype) == 'jacobi' .or. (trim(pctype) == 'gamg' .and. trim(ksptype) == 'cg'))
  end function gpu_petsc_solve_supported

  subroutine gpu_petsc_solve_scalar(x, matrix, rhs, option_path, iterations_taken)
    !!< petsc_solve_scalar (femtools/Solvers.F90:111) on the GPU, with the
    !!< reference's argument list (the preconditioner_matrix, prolongators,
    !!< surface_node_list and internal_smoothing_option arguments of the
    !!< reference are for the mg preconditioner, which this path does not
    !!< offer).  Inactive rows of matrix are ghost rows, as in the reference;
    !!< x holds the initial guess unless start_from_zero and the solution on
    !!< return.  Divergence is reported as ConvergenceCheck reports it.
    type(scalar_field), intent(inout), target :: x
    type(csr_matrix), intent(in), target :: matrix
    type(scalar_field), intent(in), target :: rhs
    character(len=*), optional, intent(in) :: option_path
    integer, intent(out), optional :: iterations_taken

    character(len=OPTION_PATH_LEN) :: path
    character(len=FIELD_NAME_LEN) :: ksptype, pctype
    character(len=30), dimension(10) :: reasons
    type(fl_solver_opts) :: opts
    type(fl_solve_report) :: report
    type(c_ptr) :: handle, inactive_ptr
    integer(c_int8_t), dimension(:), allocatable, target :: inactive
    integer :: restart, max_its, n
    real :: rtol, atol

    if (present(option_path)) then
       path = solver_path(option_path)
    else
       path = solver_path(x%option_path)
    end if
    call get_option(trim(path) // '/iterative_method[0]/name', ksptype)
    call get_option(trim(path) // '/preconditioner[0]/name', pctype)
    if (.not. ((trim(ksptype) == 'cg' .or. trim(ksptype) == 'gmres') .and. trim(pctype) == 'jacobi')) then
       FLAbort("gpu_petsc_solve_scalar: cg or gmres with jacobi (gamg through fl_amg_*)")
    end if
    call get_option(trim(path) // '/iterative_method::gmres/restart', restart, default=30)
    call get_option(trim(path) // '/relative_error', rtol)
    call get_option(trim(path) // '/absolute_error', atol, default=0.0)
    call get_option(trim(path) // '/max_iterations', max_its)
    opts%ksp_type = merge(0, 1, trim(ksptype) == 'cg')
    opts%restart = restart
    opts%rtol = rtol
    opts%atol = atol
    opts%dtol = 1.0e5
    opts%max_its = max_its
    opts%start_from_zero = merge(1, 0, have_option(trim(path) // '/start_from_zero'))
    opts%precision = 0
    opts%inner_rtol = 1.0e-5
    opts%norm_type = 0
    opts%schedule = 0

    n = size(matrix, 1)
    inactive_ptr = c_null_ptr
    if (associated(matrix%inactive%ptr)) then
       allocate(inactive(n))
       inactive = merge(1_c_int8_t, 0_c_int8_t, matrix%inactive%ptr(1:n))
       inactive_ptr = c_loc(inactive(1))
    end if
    handle = gpu_pattern_handle(matrix)
    call gpu_check(fl_gpu_petsc_solve(handle, opts, c_loc(matrix%val(1)), inactive_ptr, c_loc(rhs%val(1)), &
         c_loc(x%val(1)), report), "fl_gpu_petsc_solve")
    if (allocated(inactive)) deallocate(inactive)
    if (present(iterations_taken)) iterations_taken = report%iterations

    ! ConvergenceCheck (Solvers.F90:1369-1479) without the matrixdump
    if (report%reason <= 0) then
       reasons(1) = "Undefined"
       reasons(2) = "KSP_DIVERGED_NULL"
       reasons(3) = "KSP_DIVERGED_ITS"
       reasons(4) = "KSP_DIVERGED_DTOL"
       reasons(5) = "KSP_DIVERGED_BREAKDOWN"
       reasons(6) = "KSP_DIVERGED_BREAKDOWN_BICG"
       reasons(7) = "KSP_DIVERGED_NONSYMMETRIC"
       reasons(8) = "KSP_DIVERGED_INDEFINITE_PC"
       reasons(9) = "KSP_DIVERGED_NAN"
       reasons(10) = "KSP_DIVERGED_INDEFINITE_MAT"
       ewrite(-1, *) 'WARNING: Failed to converge.'
       ewrite(-1, *) "GPU solve did not converge for matrix solve of: " // trim(x%name)
       if (report%reason >= -10 .and. report%reason <= -1) then
          ewrite(-1, *) 'Reason for non-convergence: ', reasons(-report%reason)
       else
          ewrite(-1, *) 'Reason for non-convergence is undefined: ', report%reason
       end if
       ewrite(-1, *) 'Number of iterations: ', report%iterations
       if (have_option(trim(path) // '/ignore_all_solver_failures')) then
          ewrite(0, *) 'Specified ignore_all_solver_failures, therefore continuing'
       else if (report%reason /= -3 .or. have_option(trim(path) // '/never_ignore_solver_failures')) then
          ewrite(-1, *) "Sending signal to dump and finish"
          sig_int = .true.
       else if (.not. have_option(trim(path) // '/allow_non_convergence_during_spinup')) then
          ewrite(-1, *) "Sending signal to dump and finish"
          sig_int = .true.
       end if
    end if
  end subroutine gpu_petsc_solve_scalar

  subroutine gpu_solve_field_equation_cg(field_name, state, istate, dt, velocity_name, iterations_taken)
    !!< solve_field_equation_cg (Advection_Diffusion_CG.F90:127-174) with the
    !!< GPU assembly and solve: T is reset to OldT if present, the acceleration
    !!< form is assembled and solved for delta_t from zero, and T += dt delta_t.
    character(len=*), intent(in) :: field_name
    type(state_type), dimension(:), intent(inout) :: state
    integer, intent(in) :: istate
    real, intent(in) :: dt
    character(len=*), optional, intent(in) :: velocity_name
    integer, intent(out), optional :: iterations_taken

    type(csr_matrix) :: matrix
    type(scalar_field) :: delta_t, rhs
    type(scalar_field), pointer :: t, t_old
    type(csr_sparsity), pointer :: sparsity
    integer :: stat

    t => extract_scalar_field(state(istate), field_name)
    t_old => extract_scalar_field(state(istate), "Old" // field_name, stat=stat)
    if (stat == 0) call set(t, t_old)
    sparsity => get_csr_sparsity_firstorder(state(istate), t%mesh, t%mesh)
    call allocate(matrix, sparsity, name="AdvectionDiffusionCGMatrix")
    call allocate(rhs, t%mesh, name="AdvectionDiffusionCGRHS")
    call allocate(delta_t, t%mesh, name=trim(field_name) // "Change")
    call zero(delta_t)
    call gpu_assemble_advection_diffusion_cg(t, matrix, rhs, state(istate), dt, velocity_name=velocity_name)
    call gpu_petsc_solve_scalar(delta_t, matrix, rhs, option_path=t%option_path, &
         iterations_taken=iterations_taken)
    call addto(t, delta_t, dt)
    call deallocate(matrix)
    call deallocate(rhs)
    call deallocate(delta_t)
  end subroutine gpu_solve_field_equation_cg

end module fl_gpu_bindings
