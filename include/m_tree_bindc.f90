! m_tree_bindc.f90 -- Fortran interface to libtree2d_gb300.so.
!
! Drop-in for the reference's binding module (ver-c/src/m_tree_bindc.f90:1-17):
! same module name, same procedure names, same argument passing -- nvor_b, x
! and y by value, arrays and u, v by reference, vor_b(2,nvor_b) holding x,y
! per blob (the C side sees double[nvor_b][2]).  A solver that does
!     use m_tree_bindc
!     call make_tree(nvor_b, vor_b, cir_b, cor_b)
!     call biot_tree(x1, y1, u3, v3)
! links against libtree2d_gb300.so instead of the reference objects and
! needs no other change.  The extra interfaces below are optional.
module m_tree_bindc
  use, intrinsic :: iso_c_binding
  implicit none

  interface
    subroutine make_tree(nvor_b, vor_b, cir_b, cor_b) bind(c, name="make_tree")
      import :: c_int, c_double
      integer(c_int), value, intent(in) :: nvor_b
      real(c_double), intent(in) :: vor_b(2, nvor_b), cir_b(nvor_b), cor_b(nvor_b)
    end subroutine make_tree

    subroutine biot_tree(x, y, u, v) bind(c, name="biot_tree")
      import :: c_double
      real(c_double), value, intent(in) :: x, y
      real(c_double), intent(out) :: u, v
    end subroutine biot_tree

    ! Optional: all points of a loop in one call (uv(2,n) receives u,v).
    integer(c_int) function biot_tree_batch(n, xy, uv) bind(c, name="biot_tree_batch")
      import :: c_int, c_double
      integer(c_int), value, intent(in) :: n
      real(c_double), intent(in) :: xy(2, n)
      real(c_double), intent(out) :: uv(2, n)
    end function biot_tree_batch

    ! Optional: parameters without ../cal_cond/fmm_param.dat.
    integer(c_int) function tree2d_set_params(nterms, num_p, theta, r_min) bind(c, name="tree2d_set_params")
      import :: c_int, c_double
      integer(c_int), value, intent(in) :: nterms, num_p
      real(c_double), value, intent(in) :: theta, r_min
    end function tree2d_set_params

    ! Optional: 0 = plain FP64 (default), 1 = mixed precision, 2 = learned order.
    integer(c_int) function tree2d_set_mode(mode) bind(c, name="tree2d_set_mode")
      import :: c_int
      integer(c_int), value, intent(in) :: mode
    end function tree2d_set_mode

    ! Optional: status of the last call (0 = ok).
    integer(c_int) function tree2d_last_error() bind(c, name="tree2d_last_error")
      import :: c_int
    end function tree2d_last_error

    ! Optional: load a network for the learned mode from its raw weights
    ! file; path ends in a NUL, e.g. trim(dir)//"/learned_weights.t2dw"//c_null_char.
    integer(c_int) function tree2d_learn_load(path) bind(c, name="tree2d_learn_load")
      import :: c_int, c_char
      character(kind=c_char), dimension(*), intent(in) :: path
    end function tree2d_learn_load
  end interface
end module m_tree_bindc
