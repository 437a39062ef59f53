"""Generate the golden fixtures in this folder by running jclsquant itself.

The reference is imported from its source tree with its Cython kernels
compiled from the reference .pyx sources (oracle/reference_import.py); this
script therefore runs only where that tree exists.  The committed .npz files
are what the tests read.

Every case feeds the reference's own objects (ell_matrix built from CSR by
its csr_to_ell / data_indices_c, its bounds(), modifier_bounds, rec_A_tab,
...) and stores its inputs (the reference's padded ELL arrays) and outputs.
The largest case (64 x 64 honeycomb cells, the CPU-runnable DOS
configuration) stores only outputs plus a digest of the inputs, which the
tests rebuild with minijclsquant_gb300.lattice.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import reference_import  # noqa: E402

from minijclsquant_gb300 import lattice  # noqa: E402


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("wrote %s (%d bytes)" % (path, os.path.getsize(path)))


def moments_case(ref, name, H, M, seeds, extra=None, store_inputs=True, dos=True):
    rf = ref.recurrence_functions
    H_kpm = H.modifier(ref.modifiers.modifier_bounds)
    n = int(H.shape[0])
    vs = np.stack([ref.observables.random_vector_generator(n, s) for s in seeds])
    mus = np.stack([rf.rec_A_tab(M, H_kpm, v) for v in vs])
    out = dict(M=np.int64(M), seeds=np.asarray(seeds), bounds=np.asarray(H.bounds), mu=mus, len_row=np.int64(H.len_row),
               n=np.int64(n))
    if store_inputs:
        out.update(data=H.data, indices=H.indices, valid=H.valid_row_values, data_kpm=H_kpm.data, v=vs)
    else:
        out.update(input_digest=np.array(digest(H.data, H.indices)), kpm_digest=np.array(digest(H_kpm.data)))
    if dos:
        out["dos"] = ref.observables.kpm_dos(H, M, vs[0])
    if extra:
        out.update(extra)
    save(name, **out)
    return H, H_kpm, vs


def main():
    ref = reference_import.load()
    rf = ref.recurrence_functions
    km = ref.kernel_and_moments

    # 1. builder honeycomb, 8 x 8 cells (128 sites), W = 0.5, periodic: moments, two-vector
    #    moments, series, commutator series and the time-domain Kubo correlator.
    arr = lattice.honeycomb_arrays(8, 8, t=-2.7, W=0.5, seed=1234)
    csr = lattice.to_csr(arr)
    dx = lattice.to_csr(dict(arr, data=arr["dx"]))
    dy = lattice.to_csr(dict(arr, data=arr["dy"]))
    H = ref.ell_matrix.ell_matrix(csr, dx, dy, None)
    H, H_kpm, vs = moments_case(ref, "honeycomb_8x8", H, 64, [1000, 1001])
    n = int(H.shape[0])
    v_l = ref.observables.random_vector_generator(n, 77)
    mu_lr = rf.rec_A_tab2v(64, H_kpm, v_l, vs[0])
    mu_a, mu_b = rf.rec_A_tab2v_2(64, H_kpm, v_l, vs[0])
    coef = (km.moments_FD_T0(0.1, 48) * km.JacksonKernel(48)).astype(np.complex128)
    series = rf.rec_A_vec(48, H_kpm, coef, vs[0])
    V2 = H.modifier(ref.modifiers.modifier_velocity_bounds, "x")
    V1 = H.modifier(ref.modifiers.modifier_velocity, "y")
    comm = rf.rec_com_A_vec(48, H_kpm, V2, coef, vs[0])
    # time-domain Kubo, the CPU loop of kpm_sigma_time (historical observables),
    # restated with the reference's own rec_com_A_vec / rec_A_vec / aAxby / vdot:
    M2 = 12
    cu = km.moments_U(0.8, M2)
    len_t = 4
    sig = np.zeros(len_t, dtype=np.complex128)
    aux = np.zeros(n, dtype=np.complex128)
    U = vs[0].copy()
    Uc = rf.rec_com_A_vec(48, H_kpm, V2, coef, vs[0])
    for j in range(len_t):
        if j > 0:
            U = rf.rec_A_vec(M2, H_kpm, cu, U)
            Uc = rf.rec_A_vec(M2, H_kpm, cu, Uc)
        V1.dot(1.0 + 0j, 0 + 0j, U, aux)
        sig[j] = ref.blas_funs.vdot(1 + 0j, Uc, aux, n, H.n_threads)
    save("honeycomb_8x8_more", v_l=v_l, mu_lr=mu_lr, mu2_a=mu_a, mu2_b=mu_b, coef=coef, series=series,
         v2_data=V2.data, v1_data=V1.data, comm=comm, cu=cu, sigma=sig, M2=np.int64(M2), len_t=np.int64(len_t),
         dx_vec=H.dx_vec, dy_vec=H.dy_vec)

    # 2. the reference's own graphene builder (non-Hermitian 1e-6 (Dx+Dy) term), 256 sites
    np.random.seed(5)
    S = ref.lattice.lattice_hexagonal(256)
    Hg = ref.hams.H_graphene(S, -2.7 + 0j, 0, 0.5, True, "ELL")
    moments_case(ref, "ref_graphene_256", Hg, 128, [11, 12])

    # 3. complex hoppings (Peierls-like phase on every bond), 6 x 6 cells, open boundaries
    arr = lattice.honeycomb_arrays(6, 5, t=-2.7, W=0.3, seed=9, periodic=False)
    phase = np.exp(1j * 0.7 * np.real(arr["dx"]) / 0.142)
    arr_c = dict(arr, data=np.where(np.real(arr["dx"]) != 0, arr["data"] * phase, arr["data"]))
    Hc = ref.ell_matrix.ell_matrix(lattice.to_csr(arr_c))
    moments_case(ref, "complex_open_6x5", Hc, 96, [3])

    # 4. irregular sparse matrix: each row adds 0..3 random Hermitian bond pairs plus a real
    #    diagonal, so row lengths vary and padding uses the last valid column
    rng = np.random.default_rng(2024)
    nr = 300
    rows, cols, vals = [], [], []
    for i in range(nr):
        k = rng.integers(0, 4)
        for j in rng.choice(nr, size=k, replace=False):
            if j == i:
                continue
            w = rng.normal() + 1j * rng.normal()
            rows += [i, j]
            cols += [j, i]
            vals += [w, np.conj(w)]
        rows.append(i)
        cols.append(i)
        vals.append(rng.normal())
    import scipy.sparse as sp

    Hr = sp.csr_matrix((vals, (rows, cols)), shape=(nr, nr))
    Hr.sum_duplicates()
    Hi = ref.ell_matrix.ell_matrix(Hr.tocsr())
    moments_case(ref, "irregular_300", Hi, 80, [21, 22, 23])

    # 5. tiny edge cases: 2 x 2 cells (8 sites) with M = 1, 2 and 3
    arr = lattice.honeycomb_arrays(2, 2, t=-1.0, W=0.2, seed=1)
    Ht = ref.ell_matrix.ell_matrix(lattice.to_csr(arr))
    Htk = Ht.modifier(ref.modifiers.modifier_bounds)
    v = ref.observables.random_vector_generator(8, 5)
    # M = 1 is an error in the reference (rec_A_tab writes A_vec[1]): record the exception type.
    try:
        rf.rec_A_tab(1, Htk, v)
        m1_error = ""
    except Exception as exc:  # the reference raises IndexError
        m1_error = type(exc).__name__
    save("tiny_2x2", data=Ht.data, indices=Ht.indices, valid=Ht.valid_row_values, data_kpm=Htk.data,
         bounds=Ht.bounds, len_row=np.int64(Ht.len_row), n=np.int64(8), v=v, m1_error=np.array(m1_error),
         mu2=rf.rec_A_tab(2, Htk, v), mu3=rf.rec_A_tab(3, Htk, v))

    # 6. the CPU-runnable DOS configuration: 64 x 64 cells = 8192 sites, W = 0.5 (seed 1234),
    #    M = 512, R = 4 vectors (seeds 1000..1003).  Inputs are rebuilt by the tests.
    arr = lattice.honeycomb_arrays(64, 64, t=-2.7, W=0.5, seed=1234)
    H64 = ref.ell_matrix.ell_matrix(lattice.to_csr(arr))
    moments_case(ref, "honeycomb_64x64", H64, 512, [1000, 1001, 1002, 1003], store_inputs=False)

    # 7. analytic kernel / moment functions of the reference
    E = np.linspace(-0.99, 0.99, 7)
    save("kernels", jackson_64=km.JacksonKernel(64), jackson_512=km.JacksonKernel(512), E=E,
         delta=np.stack([km.moments_delta(e, 32) for e in E]), fd_t0=np.stack([km.moments_FD_T0(e, 32) for e in E]),
         mu_U=km.moments_U(1.3, 40), gmas=np.stack([km.moments_Gmas(e, 16) for e in E]))

    time_evolution_case(ref)
    modifiers_case(ref)
    commutator_table_case(ref)
    two_vector_dos_case(ref)
    kernels_more_case(ref)


def time_evolution_case(ref):
    """8. time evolution (for_time, jclsquant/cuda_cython/cuda/obv.cu:93-122): len_t times
    U <- sum_m c_m T_m U and U_c <- sum_m c_m T_m U_c with the time-step moments of
    exp(-i H dt).  The device rec_A it calls (recursions.cu:267-317) is the recursion of
    the reference's CPU rec_A_vec (recurrence_functions.py:114-143), which runs here.
    The operator has complex (Peierls-like) hoppings and open boundaries."""
    rf = ref.recurrence_functions
    km = ref.kernel_and_moments
    arr = lattice.honeycomb_arrays(6, 5, t=-2.7, W=0.4, seed=31, periodic=False)
    phase = np.exp(1j * 0.5 * np.real(arr["dx"]) / 0.142)
    arr_c = dict(arr, data=np.where(np.real(arr["dx"]) != 0, arr["data"] * phase, arr["data"]))
    H = ref.ell_matrix.ell_matrix(lattice.to_csr(arr_c))
    H_kpm = H.modifier(ref.modifiers.modifier_bounds)
    n = int(H.shape[0])
    M, len_t, dt = 24, 5, 0.9
    c = km.moments_U(dt, M).astype(np.complex128)
    U0 = ref.observables.random_vector_generator(n, 501)
    Uc0 = ref.observables.random_vector_generator(n, 502)
    U, Uc = U0.copy(), Uc0.copy()
    for _ in range(len_t):
        U = rf.rec_A_vec(M, H_kpm, c, U)
        Uc = rf.rec_A_vec(M, H_kpm, c, Uc)
    save("time_evolution_6x5", data_kpm=H_kpm.data, indices=H.indices, len_row=np.int64(H.len_row),
         n=np.int64(n), c=c, M=np.int64(M), len_t=np.int64(len_t), U0=U0, Uc0=Uc0, U=U, Uc=Uc)


def modifiers_case(ref):
    """9. time-dependent operators of driven systems: the reference's own light modifier
    (light_modifier_cython, jclsquant/cython_modules/Extra_funs.pyx:236-342) in its four
    forms and its phonon modifier (hopping_pos_phonons_modifier, Extra_funs.pyx:540-560),
    on graphene ELL arrays with bond vectors (jclsquant's ell_matrix from CSR)."""
    m = ref.modifiers
    arr = lattice.honeycomb_arrays(6, 5, t=-2.7, W=0.3, seed=7)
    dx = lattice.to_csr(dict(arr, data=arr["dx"]))
    dy = lattice.to_csr(dict(arr, data=arr["dy"]))
    H = ref.ell_matrix.ell_matrix(lattice.to_csr(arr), dx, dy, None)
    size = len(H.data)
    out = dict(data=H.data, indices=H.indices, len_row=np.int64(H.len_row), dx=H.dx_vec, dy=H.dy_vec)
    # (a, A0, t, w, Tp, eta): linear, circular (right), linear packed, circular packed (left), complex A0
    light = np.array([[1, 2.1, 0.37, 1.9, 0, 0], [1, 2.1, 0.37, 1.9, 0, 1], [1, 1.4, 0.9, 2.3, 0.6, 0],
                      [1, 1.4, 0.9, 2.3, 0.6, -1], [0.5 + 0.2j, 0.7 + 0.05j, 1.1, 0.8, 0.3, 1]], dtype=np.complex128)
    light_out = []
    for a, A0, t, w, Tp, eta in light:
        new = np.zeros(size, dtype=np.complex128)
        m.light_modifier_cython(a, A0, t, w, Tp, eta, H.data, H.dx_vec, H.dy_vec, new, size, 2)
        light_out.append(new)
    out.update(light_params=light, light_out=np.stack(light_out))
    # phonons: the 'chiral_+' polarisation of modifier_hoppings_c_r (jclsquant/modifiers.py:417-421)
    n = int(H.shape[0])
    a0, b, Aq, wq, t = 0.142 + 0j, 3.37 + 0j, 0.01 + 0j, 2.0 + 0j, 0.8 + 0j
    q = np.array([4 * np.pi / (3 * np.sqrt(3) * 0.142), 0], dtype=np.complex128)
    ex = np.ascontiguousarray(np.array([1 / np.sqrt(2), 1 / np.sqrt(2)] * (n // 2), dtype=np.complex128))
    ey = np.ascontiguousarray(np.array([1j / np.sqrt(2), -1j / np.sqrt(2)] * (n // 2), dtype=np.complex128))
    rng = np.random.default_rng(11)
    S = rng.uniform(0, 2.0, (n, 2)).astype(np.complex128)
    d_new, dx_new, dy_new = H.data.copy(), H.dx_vec.copy(), H.dy_vec.copy()
    m.hopping_pos_phonons_modifier(H.data, H.indices, H.dx_vec, H.dy_vec, d_new, dx_new, dy_new, a0, b, Aq, ex, ey,
                                   wq, t, np.ascontiguousarray(S[:, 0]), np.ascontiguousarray(S[:, 1]), q, H.len_row,
                                   size, 2)
    out.update(phonon_params=np.array([a0, b, Aq, wq, t, q[0], q[1]]), e_pol_x=ex, e_pol_y=ey,
               Sx=np.ascontiguousarray(S[:, 0]), Sy=np.ascontiguousarray(S[:, 1]), phonon_data=d_new,
               phonon_dx=dx_new, phonon_dy=dy_new)
    save("modifiers_6x5", **out)


def commutator_table_case(ref):
    """10. the commutator table rec_com_A_vec_tab (jclsquant/recurrence_functions.py:202-250):
    C_tab[m] = c_m C_m on a graphene lattice with complex (Peierls-like) hoppings and open
    edges, V the rescaled velocity H o dx / a (modifier_velocity_bounds)."""
    rf = ref.recurrence_functions
    km = ref.kernel_and_moments
    arr = lattice.honeycomb_arrays(5, 4, t=-2.7, W=0.6, seed=17, periodic=False)
    phase = np.exp(1j * 0.4 * np.real(arr["dy"]) / 0.142)
    arr_c = dict(arr, data=np.where(np.real(arr["dy"]) != 0, arr["data"] * phase, arr["data"]))
    dx = lattice.to_csr(dict(arr, data=arr["dx"]))
    dy = lattice.to_csr(dict(arr, data=arr["dy"]))
    H = ref.ell_matrix.ell_matrix(lattice.to_csr(arr_c), dx, dy, None)
    H_kpm = H.modifier(ref.modifiers.modifier_bounds)
    V = H.modifier(ref.modifiers.modifier_velocity_bounds, "x")
    n = int(H.shape[0])
    M = 20
    coef = (km.moments_FD_T0(-0.2, M) * km.JacksonKernel(M)).astype(np.complex128)
    v = ref.observables.random_vector_generator(n, 808)
    tab = rf.rec_com_A_vec_tab(M, H_kpm, V, coef, v)
    save("commutator_table_5x4", data_kpm=H_kpm.data, v_data=V.data, indices=H.indices, len_row=np.int64(H.len_row),
         n=np.int64(n), M=np.int64(M), coef=coef, v=v, tab=tab, series=rf.rec_com_A_vec(M, H_kpm, V, coef, v))


def two_vector_dos_case(ref):
    """11. the two-vector DOS kpm_n_dos_n (jclsquant/observables.py:59-120) with and without
    a projector (an ELL matrix applied to the bra vector by its .dot), with bounds=True and
    bounds=False (H already rescaled).  kpm_dos_2_gpu (jclsquant/observables_gpu.py:46-93)
    computes the same quantity through the device recursion of the same maths, so these
    outputs pin both entry points."""
    ob = ref.observables
    arr = lattice.honeycomb_arrays(8, 8, t=-2.7, W=0.5, seed=1234)
    H = ref.ell_matrix.ell_matrix(lattice.to_csr(arr))
    n = int(H.shape[0])
    M = 64
    v_l = ob.random_vector_generator(n, 31)
    v_r = ob.random_vector_generator(n, 32)
    import scipy.sparse as sp

    # projector on sublattice A (even sites), weighted 0.5..1.5 per site
    w = np.where(np.arange(n) % 2 == 0, 0.5 + np.linspace(0, 1, n), 0.0).astype(np.complex128)
    P = ref.ell_matrix.ell_matrix(sp.csr_matrix(sp.diags(w)).tocsr())
    plain = ob.kpm_n_dos_n(H, M, v_l, v_r)
    proj = ob.kpm_n_dos_n(H, M, v_l, v_r, True, P)
    H_kpm = H.modifier(ref.modifiers.modifier_bounds)
    # bounds=False: the caller passes the rescaled operator (with the original bounds kept
    # on the object for the energy grid, as the reference reads H.bounds)
    H_kpm.bounds = H.bounds
    nob = ob.kpm_n_dos_n(H_kpm, M, v_l, v_r, False)
    save("two_vector_dos_8x8", data=H.data, indices=H.indices, valid=H.valid_row_values, bounds=np.asarray(H.bounds),
         len_row=np.int64(H.len_row), n=np.int64(n), M=np.int64(M), v_l=v_l, v_r=v_r, proj_data=P.data,
         proj_indices=P.indices, proj_len_row=np.int64(P.len_row), dos=plain, dos_proj=proj, dos_nobounds=nob)


def kernels_more_case(ref):
    """12. the broadened Green's function and delta moments and the tabulated Fermi-Dirac
    moments (jclsquant/kernel_and_moments.py:33-44, 107-115)."""
    km = ref.kernel_and_moments
    E = np.linspace(-0.95, 0.95, 5)
    eta = np.array([1e-3, 0.02, 0.1])
    g2 = np.stack([np.stack([km.moments_Gmas_2(e, b, 48) for b in eta]) for e in E])
    d2 = np.stack([np.stack([km.moments_delta_2(e, b, 48) for b in eta]) for e in E])
    grid = np.linspace(-1 + 1e-3, 1 - 1e-3, 401)
    fd_tab = np.stack([1 / (1 + np.exp((grid - ef) / kt)) for ef, kt in ((0.0, 0.02), (-0.3, 0.1), (0.6, 0.005))])
    fd = np.stack([km.moments_FD(64, f) for f in fd_tab])
    save("kernels_more", E=E, eta=eta, gmas2=g2, delta2=d2, fd_tab=fd_tab, moments_fd=fd)


CASES = {"time_evolution_6x5": time_evolution_case, "modifiers_6x5": modifiers_case,
         "commutator_table_5x4": commutator_table_case, "two_vector_dos_8x8": two_vector_dos_case,
         "kernels_more": kernels_more_case}


if __name__ == "__main__":
    # With case names as arguments only those cases are rewritten; with none, all of them.
    if len(sys.argv) > 1:
        for name in sys.argv[1:]:
            CASES[name](reference_import.load())
    else:
        main()
