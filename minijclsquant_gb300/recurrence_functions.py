"""Chebyshev recursions, drop-in for jclsquant/recurrence_functions.py.

Same names, argument order, defaults and return values; every recursion runs
as the fused sm_103a kernel of libkpm on the operator's cached device copy.
Extras are keyword-only: ``dtype`` ('c128' — the drop-in form — or 'c64',
complex64 recursion with FP64 moment accumulation).  Vector arguments may be
one vector [N] (reference behaviour) or R vectors [R, N] advanced together;
numpy in gives numpy out, CUDA tensors in give CUDA tensors out.
Missing-argument behaviour matches the reference (message, then None); strict mode
(``errors.set_strict(True)`` or KPM_STRICT_ERRORS=1) raises ValueError instead.
"""
from __future__ import annotations

from . import device, errors


def _check_order(M):
    # The reference writes A_vec[1] unconditionally, so M < 2 ends in an IndexError there.
    if int(M) < 2:
        raise IndexError("index 1 is out of bounds for axis 0 with size %d (M must be >= 2)" % int(M))


def rec_A_tab(M, A, v=None, *, dtype="c128"):
    """mu_m = <v | T_m(A) v>, m < M (jclsquant/recurrence_functions.py:9-40)."""
    if v is None:
        return errors.missing("You must introduce a vector.")
    _check_order(M)
    return device.cheb_moments(A.device(), M, v, dtype=dtype)


def rec_A_tab2v(M, A, v_l=None, v_r=None, *, dtype="c128"):
    """mu_m = <v_l | T_m(A) v_r> (jclsquant/recurrence_functions.py:44-74)."""
    if v_r is None or v_l is None:
        return errors.missing("You must introduce a right and left vector.")
    _check_order(M)
    return device.cheb_moments(A.device(), M, v_r, v_l=v_l, dtype=dtype)


def rec_A_tab2v_2(M, A, v_l=None, v_r=None, *, dtype="c128"):
    """(<v_l|T_m v_r>, <v_r|T_m v_r>) from one recursion (jclsquant/recurrence_functions.py:76-111)."""
    if v_r is None or v_l is None:
        return errors.missing("You must introduce a right and left vector.")
    _check_order(M)
    return device.cheb_moments(A.device(), M, v_r, v_l=v_l, dtype=dtype, both=True)


def rec_A_vec(M, A, moments_kernel=None, v=None, *, dtype="c128"):
    """sum_m c_m T_m(A) v (jclsquant/recurrence_functions.py:114-143)."""
    if moments_kernel is None:
        return errors.missing("You must introduce the analytical_moments*Kernel which is an array of size M")
    if v is None:
        return errors.missing("You must introduce a vector.")
    return device.cheb_series(A.device(), M, moments_kernel, v, dtype=dtype)


def rec_com_A_vec(M, A, V=None, moments_kernel=None, v=None):
    """Commutator series sum_m c_m C_m (jclsquant/recurrence_functions.py:146-196)."""
    if V is None:
        return errors.missing("You must introduce kpm renormalized velocity .")
    if moments_kernel is None:
        return errors.missing("You must introduce the analytical_moments*Kernel which is an array of size M .")
    if v is None:
        return errors.missing("You must introduce a vector.")
    return device.cheb_commutator_series(A.device(), V.device(), M, moments_kernel, v)


def rec_com_A_vec_tab(M, A, V=None, moments_kernel=None, v=None):
    """Table of the commutator series, C_tab[m] = c_m C_m, an [M, N] array
    (jclsquant/recurrence_functions.py:202-250); [R, M, N] for R vectors."""
    if V is None:
        return errors.missing("You must introduce kpm renormalized velocity .")
    if v is None:
        return errors.missing("You must introduce a vector.")
    if moments_kernel is None:
        # the reference indexes moments_kernel[0] unconditionally
        raise TypeError("'NoneType' object is not subscriptable")
    _check_order(M)
    return device.cheb_commutator_table(A.device(), V.device(), M, moments_kernel, v)
