"""GB300-native GFN2-xTB trajectory-step engine for QCxMS.

The compute path is ``libqcxgpu.so`` (hand-written sm_103a CUDA kernels behind
the C ABI in ``include/qcxgpu.h``). This package only binds that ABI with
ctypes and mirrors the reference's Fortran interface:

* :func:`get_xtb_egrad` -- ``module qcxms_tblite``'s ``get_xtb_egrad``
  (``src/tblite.f90:65-175``): atomic numbers, Bohr coordinates, charge,
  multiplicity, method and electronic temperature in; charges, energy,
  gradient and a status code out.
* :class:`Batch` -- many trajectories advanced together (leapfrog of
  ``src/md.f90:749-773`` followed by the energy/gradient call, as in the MD
  loop at ``src/md.f90:390-396``).
* :func:`fragment_ips` / :func:`boltz` -- the GFN2 fragment IPs of ``analyse``
  (``src/analyse.f90:13-467``) for many fragmented structures in one batch,
  and ``boltz`` (``src/utility.f90:469-498``).

There is no CPU fallback: if the CUDA library cannot be loaded, every call
raises.
"""
import ctypes
import os

import numpy as np

from . import constants

__all__ = ["gfn1_xtb", "gfn2_xtb", "ipea1_xtb", "get_xtb_egrad", "Batch", "fragment_ips", "fragment_formula", "boltz", "read_ensemble", "load_library",
           "library_path",
           "STATUS_SCC_NOT_CONVERGED", "STATUS_NON_FINITE", "STATUS_CHOLESKY_FAILED", "STATUS_EIGEN_NOT_CONVERGED",
           "STATUS_CHECKQC", "checkqc"]

# method selectors, src/tblite.f90:34-40
gfn1_xtb = 1
gfn2_xtb = 2
ipea1_xtb = 11

STATUS_SCC_NOT_CONVERGED = 1
STATUS_NON_FINITE = 2
STATUS_CHOLESKY_FAILED = 4
STATUS_EIGEN_NOT_CONVERGED = 8
STATUS_CHECKQC = 16
STATUS_SCC_PENDING = 32

_HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def library_path():
    return os.path.join(_HERE, "_build", "libqcxgpu.so")


def load_library(build_if_missing=True):
    """Load libqcxgpu.so (building it in-tree first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if build_if_missing:
        from . import build as _build
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libqcxgpu.so is missing (%s); run __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    c_int, c_double, c_ll = ctypes.c_int, ctypes.c_double, ctypes.c_longlong
    P = ctypes.POINTER
    lib.qcx_version.restype = c_int
    lib.qcx_last_error.restype = ctypes.c_char_p
    lib.qcx_egrad.restype = c_int
    lib.qcx_egrad.argtypes = [c_int, c_int, P(ctypes.c_int32), P(c_double), c_int, c_int, c_double,
                              P(c_double), P(c_double), P(c_double)]
    lib.qcx_batch_create.restype = ctypes.c_void_p
    lib.qcx_batch_create.argtypes = [c_int, P(ctypes.c_int32), P(ctypes.c_int32), P(c_double), P(c_double)]
    lib.qcx_batch_destroy.argtypes = [ctypes.c_void_p]
    lib.qcx_batch_set_scc.argtypes = [ctypes.c_void_p, c_int, c_double, c_double, c_double]
    lib.qcx_batch_set_state.argtypes = [ctypes.c_void_p, P(c_double), P(c_double), P(c_double)]
    lib.qcx_batch_egrad.argtypes = [ctypes.c_void_p]
    lib.qcx_batch_set_timing.argtypes = [ctypes.c_void_p, c_int]
    lib.qcx_batch_get_timing.argtypes = [ctypes.c_void_p, P(ctypes.c_float), c_int]
    lib.qcx_mma_selftest.argtypes = [c_int, c_int, c_int, P(ctypes.c_float), c_int, P(ctypes.c_float), c_int,
                                     P(ctypes.c_float), c_int, P(ctypes.c_float)]
    lib.qcx_jacobi32_selftest.argtypes = [c_int, P(ctypes.c_float), P(ctypes.c_float), P(ctypes.c_float), c_int,
                                          c_double, c_int, P(c_int)]
    lib.qcx_checkqc.argtypes = [c_int, P(c_double), P(c_double), c_int, P(c_double)]
    lib.qcx_batch_load_state.argtypes = [ctypes.c_void_p, P(c_double), P(c_double)]
    lib.qcx_batch_step.argtypes = [ctypes.c_void_p, c_int, c_double]
    lib.qcx_batch_get.argtypes = [ctypes.c_void_p] + [P(c_double)] * 6 + [P(ctypes.c_int32)] * 2
    lib.qcx_batch_get_energy_terms.argtypes = [ctypes.c_void_p, c_int, P(c_double)]
    lib.qcx_batch_get_matrix.argtypes = [ctypes.c_void_p, c_int, c_int, P(c_double)]
    lib.qcx_batch_kernel_launches.restype = c_ll
    lib.qcx_batch_kernel_launches.argtypes = [ctypes.c_void_p]
    lib.qcx_batch_sync.argtypes = [ctypes.c_void_p]
    lib.qcx_batch_set_precision.argtypes = [ctypes.c_void_p, c_int]
    lib.qcx_batch_set_guess.argtypes = [ctypes.c_void_p, c_int]
    lib.qcx_batch_fragments.argtypes = [ctypes.c_void_p, ctypes.c_double, c_int, c_int, P(ctypes.c_int32),
                                        P(ctypes.c_int32)]
    lib.qcx_batch_get_progress.argtypes = [ctypes.c_void_p, P(ctypes.c_int32), P(ctypes.c_int64)]
    lib.qcx_batch_stream.restype = ctypes.c_void_p
    lib.qcx_batch_stream.argtypes = [ctypes.c_void_p]
    lib.qcx_batch_profile_egrad.argtypes = [ctypes.c_void_p, P(ctypes.c_float)]
    lib.qcx_batch_get_sizes.argtypes = [ctypes.c_void_p, P(ctypes.c_int32), P(ctypes.c_int32)]
    lib.qcx_fragment_ips.argtypes = [c_int, c_int, P(ctypes.c_int32), P(ctypes.c_int32), P(c_double),
                                     P(ctypes.c_int32), c_int, c_double, c_int, P(c_double), P(c_double),
                                     P(ctypes.c_int32)]
    lib.qcx_batch_get_md_avg_xyz.argtypes = [ctypes.c_void_p, P(c_double)]
    lib.qcx_batch_set_cid_rules.argtypes = [ctypes.c_void_p, c_double, c_int]
    lib.qcx_batch_get_cid_avg_xyz.argtypes = [ctypes.c_void_p, P(c_double)]
    lib.qcx_batch_get_cid_state.argtypes = [ctypes.c_void_p] + [P(ctypes.c_int32)] * 7 + [P(c_double)] * 2
    lib.qcx_batch_set_md_heating.argtypes = [ctypes.c_void_p, P(c_double), P(c_double), P(c_double), c_double]
    lib.qcx_batch_set_md_etemp.argtypes = [ctypes.c_void_p, c_double, c_double]
    lib.qcx_batch_get_md_etemp.argtypes = [ctypes.c_void_p, P(c_double)]
    lib.qcx_batch_set_md_rules.argtypes = [ctypes.c_void_p, c_int, c_int, c_int]
    lib.qcx_batch_get_md_state.argtypes = [ctypes.c_void_p] + [P(ctypes.c_int32)] * 5 + [P(c_double)] * 3
    lib.qcx_read_xyz.argtypes = [ctypes.c_char_p, c_int, P(ctypes.c_int32), P(ctypes.c_int32), P(c_double)]
    lib.qcx_read_start.argtypes = [ctypes.c_char_p, c_int, P(ctypes.c_int32), P(c_double), P(c_double),
                                   P(c_double), P(c_double)]
    lib.qcx_write_start.argtypes = [ctypes.c_char_p, c_int, c_int, c_double, c_double, P(c_double), P(c_double)]
    lib.qcx_fragment_formula.argtypes = [c_int, P(ctypes.c_int32), P(ctypes.c_int32), P(c_double),
                                         P(ctypes.c_int32), P(c_double), ctypes.c_char_p]
    lib.qcx_write_gs.argtypes = [ctypes.c_char_p, c_int, c_int, c_int, P(c_double), P(c_double)]
    lib.qcx_format_res.argtypes = [c_int, c_double, c_int, c_int, c_int, c_int, c_int, c_int, P(ctypes.c_int32),
                                   P(ctypes.c_int32), ctypes.c_char_p, c_int]
    lib.qcx_boltz.argtypes = [c_int, c_int, c_int, c_double, P(c_double), P(c_double)]
    lib.qcx_batch_set_keep_mo.argtypes = [ctypes.c_void_p, c_int]
    lib.qcx_batch_set_scc_budget.argtypes = [ctypes.c_void_p, c_int]
    lib.qcx_batch_step_groups.argtypes = [ctypes.c_void_p, P(ctypes.c_int32), c_double]
    lib.qcx_batch_step_paced.argtypes = [ctypes.c_void_p, c_int, c_double]
    lib.qcx_batch_autotune_budget.argtypes = [ctypes.c_void_p, c_double, P(ctypes.c_int32), c_int, c_int,
                                              P(c_double)]
    lib.qcx_batch_set_scc_budget_scale.argtypes = [ctypes.c_void_p, c_int]
    lib.qcx_batch_get_scc_budget.argtypes = [ctypes.c_void_p, P(ctypes.c_int32), P(ctypes.c_int32)]
    lib.qcx_batch_autotune_paced.argtypes = [ctypes.c_void_p, c_double, c_int, P(ctypes.c_int32), c_int, c_int,
                                             P(c_double)]
    lib.qcx_batch_group_info.argtypes = [ctypes.c_void_p, P(ctypes.c_int32), P(ctypes.c_int32), P(c_double)]
    lib.qcx_batch_get_iterations.argtypes = [ctypes.c_void_p, P(ctypes.c_int64)]
    lib.qcx_batch_mo_populations.argtypes = [ctypes.c_void_p, c_int, P(c_double), P(c_double), P(c_double),
                                             P(ctypes.c_int32)]
    lib.qcx_mo_spectrum.argtypes = [c_int, c_int, P(ctypes.c_int32), P(c_double), c_int, c_int, c_double,
                                    P(c_double), P(ctypes.c_int32), P(ctypes.c_int32), P(c_double), P(c_double),
                                    P(c_double), c_int]
    lib.qcx_write_qmo.argtypes = [ctypes.c_char_p, ctypes.c_char_p, c_int, c_int, c_int, P(c_double), P(c_double),
                                  P(c_double)]
    _lib = lib
    return lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _err(lib):
    return lib.qcx_last_error().decode()


def get_xtb_egrad(num, xyz, charge, multiplicity, method=gfn2_xtb, etemp=300.0, output_file=None):
    """Energy, gradient and Mulliken charges of one structure.

    Mirrors ``get_xtb_egrad`` of ``src/tblite.f90:65-175``. Returns
    ``(qat, energy, gradient, stat)`` with ``stat`` = 0 (ok), 5 (unknown or
    unsupported method) or -1 (failure). When ``output_file`` is given a
    one-line summary is written there, as the reference always (re)creates it.
    """
    lib = load_library()
    num = np.ascontiguousarray(num, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(len(num), 3)
    e = np.zeros(1)
    g = np.zeros((len(num), 3))
    q = np.zeros(len(num))
    stat = lib.qcx_egrad(int(method), len(num), _ip(num), _dp(xyz), int(charge), int(multiplicity),
                         float(etemp), _dp(e), _dp(g), _dp(q))
    if output_file:
        with open(output_file, "w") as f:
            f.write("qcxgpu GFN2-xTB energy %.12f Eh stat %d %s\n" % (e[0], stat, _err(lib) if stat else ""))
    return q, float(e[0]), g, int(stat)


MAX_FRAGMENTS = 10


def read_ensemble(root="TMPQCXMS", charge=1):
    """Every trajectory of a QCxMS ensemble directory: ``root/TMP.n/start.xyz``
    and ``root/TMP.n/qcxms.start`` (wrstart, ``src/utility.f90:321-373``), in
    the order of n. Returns a list of dicts with Z, xyz (Bohr), vel, velof,
    eimp, tadd, itrj, mass and charge, ready for :class:`Batch` and
    :meth:`Batch.set_md_heating`."""
    lib = load_library()
    dirs = []
    for name in os.listdir(root):
        if name.startswith("TMP.") and name[4:].isdigit():
            dirs.append((int(name[4:]), os.path.join(root, name)))
    mols = []
    for n, d in sorted(dirs):
        nat = np.zeros(1, dtype=np.int32)
        p = os.path.join(d, "start.xyz").encode()
        if lib.qcx_read_xyz(p, 0, _ip(nat), None, None) != 0:
            raise RuntimeError(_err(lib))
        na = int(nat[0])
        Z = np.zeros(na, dtype=np.int32)
        xyz = np.zeros((na, 3))
        if lib.qcx_read_xyz(p, na, _ip(nat), _ip(Z), _dp(xyz)) != 0:
            raise RuntimeError(_err(lib))
        itrj = np.zeros(1, dtype=np.int32)
        eimp, tadd = np.zeros(1), np.zeros(1)
        vel, velof = np.zeros((na, 3)), np.zeros(na)
        if lib.qcx_read_start(os.path.join(d, "qcxms.start").encode(), na, _ip(itrj), _dp(eimp), _dp(tadd),
                              _dp(vel), _dp(velof)) != 0:
            raise RuntimeError(_err(lib))
        mols.append({"Z": Z, "xyz": xyz, "vel": vel, "velof": velof, "eimp": float(eimp[0]), "tadd": float(tadd[0]),
                     "itrj": int(itrj[0]), "mass": np.array([constants.MASS_AU[int(z)] for z in Z]),
                     "charge": charge})
    return mols


def fragment_ips(structs, mchrg=1, etemp=300.0, precision=0, method=gfn2_xtb):
    """Fragment IPs (EAs for ``mchrg`` < 0) of fragmented structures in one batch.

    Mirrors the GFN2 path of ``analyse`` (``src/analyse.f90:13-467``):
    ``structs`` is a list of dicts with ``Z``, ``xyz`` (Bohr) and ``frag``
    (1-based fragment number per atom). Returns ``(fragip, efrag, ipok)``:
    ``fragip[t]`` is an ``(nfrag, |mchrg|)`` array in eV, ``efrag[t]`` the
    ``(nfrag, |mchrg|+1)`` energies in Eh (column 0 the neutral) and ``ipok[t]``
    a bool. Raises on invalid input or a CUDA error.
    """
    lib = load_library()
    nch = abs(int(mchrg))
    nat = np.array([len(s["Z"]) for s in structs], dtype=np.int32)
    Z = np.ascontiguousarray(np.concatenate([np.asarray(s["Z"]) for s in structs]), dtype=np.int32)
    xyz = np.ascontiguousarray(np.concatenate([np.asarray(s["xyz"], dtype=np.float64).reshape(-1, 3)
                                               for s in structs]))
    frag = np.ascontiguousarray(np.concatenate([np.asarray(s["frag"]) for s in structs]), dtype=np.int32)
    ip = np.zeros((len(structs), MAX_FRAGMENTS, max(nch, 1)))
    ef = np.zeros((len(structs), MAX_FRAGMENTS, max(nch, 1) + 1))
    ok = np.zeros(len(structs), dtype=np.int32)
    rc = lib.qcx_fragment_ips(int(method), len(structs), _ip(nat), _ip(Z), _dp(xyz), _ip(frag), int(mchrg),
                              float(etemp), int(precision), _dp(ip), _dp(ef), _ip(ok))
    if rc != 0:
        raise RuntimeError("qcx_fragment_ips returned %d: %s" % (rc, _err(lib)))
    nf = [int(np.max(s["frag"])) for s in structs]
    return [ip[t, :nf[t]] for t in range(len(structs))], [ef[t, :nf[t]] for t in range(len(structs))], ok.astype(bool)


def fragment_formula(Z, frag, mass):
    """Fragment masses (amu) and sum formulas as fragmass (src/fragments.f90:10-84)."""
    lib = load_library()
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    frag = np.ascontiguousarray(frag, dtype=np.int32)
    mass = np.ascontiguousarray(mass, dtype=np.float64)
    n = np.zeros(1, dtype=np.int32)
    fm = np.zeros(MAX_FRAGMENTS)
    buf = ctypes.create_string_buffer(80 * MAX_FRAGMENTS)
    if lib.qcx_fragment_formula(len(Z), _ip(Z), _ip(frag), _dp(mass), _ip(n), _dp(fm), buf) != 0:
        raise RuntimeError(_err(lib))
    k = int(n[0])
    return fm[:k], [buf.raw[80 * i:80 * (i + 1)].split(b"\0")[0].decode() for i in range(k)]


def write_gs(path, nmax, xyz, vel):
    """qcxms.gs of a ground-state sampling run (src/md.f90:150-153, 379-385):
    xyz and vel [nrec][nat][3] (Bohr, atomic units), one record per loop top."""
    lib = load_library()
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    vel = np.ascontiguousarray(vel, dtype=np.float64)
    if xyz.ndim == 2:
        xyz, vel = xyz[None], vel[None]
    nrec, nat = xyz.shape[0], xyz.shape[1]
    if lib.qcx_write_gs(os.fsencode(path), int(nmax), nat, nrec, _dp(xyz), _dp(vel)) != 0:
        raise RuntimeError("qcx_write_gs failed: " + _err(lib))


def format_res(fragchrg3, mchrg, itrj, isec, ifrag, Z, counts, icoll=None):
    """One qcxms.res line (src/write_fragments.f90:392-447); icoll given for
    collision runs. Z, counts: the fragment's elements in order of atomic
    number and their counts."""
    lib = load_library()
    z = np.ascontiguousarray(Z, dtype=np.int32)
    c = np.ascontiguousarray(counts, dtype=np.int32)
    buf = ctypes.create_string_buffer(256)
    n = lib.qcx_format_res(int(icoll is not None), float(fragchrg3), int(mchrg), int(itrj),
                           int(icoll or 0), int(isec), int(ifrag), len(z), _ip(z), _ip(c), buf, 256)
    if n < 0:
        raise RuntimeError("qcx_format_res failed: " + _err(lib))
    return buf.value.decode()


def mo_spectrum(num, xyz, charge=0, multiplicity=1, method=None, etemp=300.0, max_nao=None):
    """get_xtb_egrad(spec_calc=.true.) for one structure (src/tblite.f90:153-166):
    returns (energy, emo [nao] in Eh, focc [nao], qmo [nao][nat], ihomo) with
    write_qmo's populations (src/mo_energ.f90:7-80)."""
    lib = load_library()
    num = np.ascontiguousarray(num, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    nat = len(num)
    mx = int(max_nao or 9 * nat)
    e = np.zeros(1)
    n = np.zeros(1, dtype=np.int32)
    ih = np.zeros(1, dtype=np.int32)
    emo, focc, qmo = np.zeros(mx), np.zeros(mx), np.zeros(mx * nat)
    rc = lib.qcx_mo_spectrum(gfn2_xtb if method is None else int(method), nat, _ip(num), _dp(xyz), int(charge),
                             int(multiplicity), float(etemp), _dp(e), _ip(n), _ip(ih), _dp(emo), _dp(focc), _dp(qmo),
                             mx)
    if rc != 0:
        raise RuntimeError("qcx_mo_spectrum returned %d: %s" % (rc, _err(lib)))
    k = int(n[0])
    return float(e[0]), emo[:k].copy(), focc[:k].copy(), qmo[:k * nat].reshape(k, nat).copy(), int(ih[0])


def write_qmo(tmp_path, mspec_path, emo, focc, qmo, ihomo):
    """write_qmo's two files (src/mo_energ.f90:26-79): tmp.mspec (list-directed,
    read back by readpopmo) and qcxms.Mspec.tbxtb; either path may be None."""
    lib = load_library()
    emo = np.ascontiguousarray(emo, dtype=np.float64)
    focc = np.ascontiguousarray(focc, dtype=np.float64)
    qmo = np.ascontiguousarray(qmo, dtype=np.float64)
    enc = lambda p: None if p is None else os.fsencode(p)
    if lib.qcx_write_qmo(enc(tmp_path), enc(mspec_path), qmo.shape[1], qmo.shape[0], int(ihomo), _dp(emo), _dp(focc),
                         _dp(qmo)) != 0:
        raise RuntimeError("qcx_write_qmo failed: " + _err(lib))


def boltz(units, temp, ip):
    """Boltzmann weights of an ``(nfrag, mchrg)`` IP array, ``boltz`` of
    ``src/utility.f90:469-498`` (units 1: kcal/mol, 2: eV)."""
    lib = load_library()
    ip = np.asfortranarray(ip, dtype=np.float64)
    out = np.zeros_like(ip, order="F")
    rc = lib.qcx_boltz(int(units), ip.shape[0], ip.shape[1], float(temp), _dp(ip), _dp(out))
    if rc != 0:
        raise RuntimeError("qcx_boltz: %s" % _err(lib))
    return out


def mma_gemm(A, B, ta=False, tb=False, reps=1):
    """The tensor-core (tcgen05, split-TF32) product of the SCC kernel on one
    CTA: returns (C, kernel ms). A is [M][K] (or [K][M] with ta), B [K][N] (or
    [N][K] with tb)."""
    lib = load_library()
    A = np.ascontiguousarray(A, dtype=np.float32)
    B = np.ascontiguousarray(B, dtype=np.float32)
    M = A.shape[1] if ta else A.shape[0]
    K = A.shape[0] if ta else A.shape[1]
    N = B.shape[0] if tb else B.shape[1]
    C = np.zeros((M, N), dtype=np.float32)
    ms = ctypes.c_float()
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    rc = lib.qcx_mma_selftest(M, N, K, fp(A), int(ta), fp(B), int(tb), fp(C), int(reps), ctypes.byref(ms))
    if rc != 0:
        raise RuntimeError("qcx_mma_selftest returned %d: %s" % (rc, _err(lib)))
    return C, ms.value


def jacobi32(A, V=None, reltol=2e-6, max_sweeps=30):
    """The SCC kernel's FP32 eigensolver (cyclic parallel Jacobi) on one CTA.
    With V (orthonormal rows) it starts warm from that basis. Returns (rotated
    A with the eigenvalues on its diagonal, eigenvector rows, sweeps used)."""
    lib = load_library()
    A = np.ascontiguousarray(A, dtype=np.float32)
    n = A.shape[0]
    Ao = np.zeros_like(A)
    Vv = np.ascontiguousarray(np.eye(n) if V is None else V, dtype=np.float32).copy()
    sw = ctypes.c_int()
    fp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    rc = lib.qcx_jacobi32_selftest(n, fp(A), fp(Ao), fp(Vv), int(V is not None), float(reltol), int(max_sweeps),
                                   ctypes.byref(sw))
    if rc != 0:
        raise RuntimeError("qcx_jacobi32_selftest returned %d: %s" % (rc, _err(lib)))
    return Ao, Vv, sw.value


def checkqc(energy, grad, qat, charge):
    """checkqc (src/iniqm.f90:684-715) evaluated on the GPU: returns (code,
    energy) with code 0 accepted, 1 |E| < 1e-8, 2 gradient norm, 3 charges."""
    lib = load_library()
    grad = np.ascontiguousarray(grad, dtype=np.float64).reshape(-1, 3)
    qat = np.ascontiguousarray(qat, dtype=np.float64)
    e = ctypes.c_double(energy)
    code = lib.qcx_checkqc(grad.shape[0], _dp(grad), _dp(qat), int(charge), ctypes.byref(e))
    if code < 0:
        raise RuntimeError("qcx_checkqc failed: " + _err(lib))
    return code, e.value


class Batch:
    """Independent trajectories on one GPU (one molecule each)."""

    def __init__(self, mols, etemp=300.0):
        lib = load_library()
        self._lib = lib
        self.nmol = len(mols)
        self.nat = np.array([len(m["Z"]) for m in mols], dtype=np.int32)
        self.offsets = np.concatenate([[0], np.cumsum(self.nat)]).astype(np.int64)
        self.natom = int(self.offsets[-1])
        Z = np.ascontiguousarray(np.concatenate([np.asarray(m["Z"]) for m in mols]), dtype=np.int32)
        charge = np.array([float(m.get("charge", 0)) for m in mols], dtype=np.float64)
        et = np.array([float(m.get("etemp", etemp)) for m in mols], dtype=np.float64)
        self.Z = Z
        h = lib.qcx_batch_create(self.nmol, _ip(self.nat), _ip(Z), _dp(charge), _dp(et))
        if not h:
            raise RuntimeError("qcx_batch_create failed: " + _err(lib))
        self._h = ctypes.c_void_p(h)
        xyz = np.concatenate([np.asarray(m["xyz"], dtype=np.float64).reshape(-1, 3) for m in mols])
        vel = np.concatenate([np.asarray(m.get("vel", np.zeros((len(m["Z"]), 3))), dtype=np.float64).reshape(-1, 3)
                              for m in mols])
        mass = np.concatenate([np.asarray(m.get("mass", np.ones(len(m["Z"]))), dtype=np.float64) for m in mols])
        self.set_state(xyz, vel, mass)

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed: %s" % (what, _err(self._lib)))

    def set_scc(self, max_iter=250, econv=1e-7, pconv=1e-6, mixing=0.25):
        self._check(self._lib.qcx_batch_set_scc(self._h, int(max_iter), float(econv), float(pconv), float(mixing)),
                    "set_scc")

    def set_guess(self, guess):
        """0 / "zero": every SCC starts from zero moments (the reference's fresh
        wavefunction); 1 / "previous": a trajectory's SCC starts from the converged
        moments of its previous geometry."""
        g = {"zero": 0, "previous": 1}.get(guess, guess)
        self._check(self._lib.qcx_batch_set_guess(self._h, int(g)), "set_guess")

    def set_precision(self, precision):
        """0 / "fp64": FP64 SCC; 1 / "mixed": FP32 iterations, then double-float finishing iterations."""
        p = {"fp64": 0, "mixed": 1}.get(precision, precision)
        self._check(self._lib.qcx_batch_set_precision(self._h, int(p)), "set_precision")

    def set_state(self, xyz=None, vel=None, mass=None):
        c = lambda a, s: None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(s)
        xyz, vel, mass = c(xyz, (self.natom, 3)), c(vel, (self.natom, 3)), c(mass, (self.natom,))
        self._check(self._lib.qcx_batch_set_state(self._h, _dp(xyz), _dp(vel), _dp(mass)), "set_state")
        self._lib.qcx_batch_sync(self._h)

    def load_state(self, xyz=None, vel=None):
        """New coordinates/velocities for the running trajectories, without
        starting new runs (qcx_batch_load_state)."""
        c = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(self.natom, 3)
        xyz, vel = c(xyz), c(vel)
        self._check(self._lib.qcx_batch_load_state(self._h, _dp(xyz), _dp(vel)), "load_state")
        self._lib.qcx_batch_sync(self._h)

    def egrad(self):
        self._check(self._lib.qcx_batch_egrad(self._h), "egrad")

    def step(self, nsteps, tstep=0.5 * constants.FSTOAU):
        self._check(self._lib.qcx_batch_step(self._h, int(nsteps), float(tstep)), "step")

    def step_groups(self, nsteps, tstep=0.5 * constants.FSTOAU):
        """Group g (by size, 0 = largest) takes nsteps[g] MD steps, every group
        from its own graph on its own stream, concurrently."""
        n = np.ascontiguousarray(nsteps, dtype=np.int32)
        self._check(self._lib.qcx_batch_step_groups(self._h, _ip(n), float(tstep)), "step_groups")

    def step_paced(self, nsteps=1, tstep=0.5 * constants.FSTOAU):
        """The largest molecules' group takes nsteps steps, every other group as
        many as fit into the same time (measured at the previous paced call)."""
        self._check(self._lib.qcx_batch_step_paced(self._h, int(nsteps), float(tstep)), "step_paced")

    def autotune_budget(self, candidates=(0, 10, 20, 40), calls=3, tstep=0.5 * constants.FSTOAU, steps_per_call=1):
        """Pick the per-step SCC budget and its scale (each group's largest
        molecule or the batch's) with the highest completed-step rate of paced
        calls of ``steps_per_call`` steps on this batch (the measured steps are
        real MD steps; two passes over the configurations, the second in reverse
        order, against the drift of the batch's state). Returns ((chosen budget, per_group), {(budget, per_group):
        trajectory-steps/s})."""
        c = np.ascontiguousarray(candidates, dtype=np.int32)
        rates = np.zeros(2 * len(c))
        best = self._lib.qcx_batch_autotune_paced(self._h, float(tstep), int(steps_per_call), _ip(c), len(c),
                                                  int(calls), _dp(rates))
        if best < 0:
            raise RuntimeError("autotune_budget failed: " + _err(self._lib))
        it = ctypes.c_int32(); pg = ctypes.c_int32()
        self._check(self._lib.qcx_batch_get_scc_budget(self._h, ctypes.byref(it), ctypes.byref(pg)), "get_scc_budget")
        out = {}
        for k, v in enumerate(rates):
            out[(int(c[k % len(c)]), 1 if k < len(c) else 0)] = float(v)
        return (int(best), int(pg.value)), out

    def set_scc_budget_scale(self, per_group=True):
        """Scale of the SCC budget in grouped and paced steps: each group's
        largest molecule (True) or the batch's largest."""
        self._check(self._lib.qcx_batch_set_scc_budget_scale(self._h, int(bool(per_group))), "set_scc_budget_scale")

    def group_info(self):
        """(group of every molecule, step counts of the last grouped call, measured ms per step)."""
        g = np.zeros(self.nmol, dtype=np.int32)
        n = np.zeros(64, dtype=np.int32)
        t = np.zeros(64)
        ng = self._lib.qcx_batch_group_info(self._h, _ip(g), _ip(n), _dp(t))
        if ng < 0:
            raise RuntimeError("group_info failed: " + _err(self._lib))
        return g, n[:ng].copy(), t[:ng].copy()

    def iterations(self):
        """SCC iterations run so far per molecule (all launches)."""
        it = np.zeros(self.nmol, dtype=np.int64)
        self._check(self._lib.qcx_batch_get_iterations(self._h, it.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))),
                    "iterations")
        return it

    def sync(self):
        self._check(self._lib.qcx_batch_sync(self._h), "sync")

    def get(self):
        xyz = np.zeros((self.natom, 3)); vel = np.zeros((self.natom, 3)); grad = np.zeros((self.natom, 3))
        energy = np.zeros(self.nmol); qat = np.zeros(self.natom); ekin = np.zeros(self.nmol)
        status = np.zeros(self.nmol, dtype=np.int32); iters = np.zeros(self.nmol, dtype=np.int32)
        self._check(self._lib.qcx_batch_get(self._h, _dp(xyz), _dp(vel), _dp(grad), _dp(energy), _dp(qat), _dp(ekin),
                                            _ip(status), _ip(iters)), "get")
        return {"xyz": xyz, "vel": vel, "grad": grad, "energy": energy, "qat": qat, "ekin": ekin,
                "status": status, "iters": iters}

    def status_iters(self):
        """Status words and SCC iteration counts of the last evaluation only."""
        status = np.zeros(self.nmol, dtype=np.int32); iters = np.zeros(self.nmol, dtype=np.int32)
        self._check(self._lib.qcx_batch_get(self._h, None, None, None, None, None, None, _ip(status), _ip(iters)),
                    "get")
        return status, iters

    def energy_terms(self, i):
        t = np.zeros(12)
        self._check(self._lib.qcx_batch_get_energy_terms(self._h, int(i), _dp(t)), "energy_terms")
        names = ["band", "ies", "e3", "aes", "axc", "disp", "atm", "rep", "ts", "total", "efermi", "iters_fp64"]
        return dict(zip(names, t))

    def matrix(self, i, which):
        nat = int(self.nat[i])
        Zi = self.Z[self.offsets[i]:self.offsets[i] + nat]
        from .basis import nao_of
        n = nao_of(Zi)
        out = np.zeros((n, n))
        rc = self._lib.qcx_batch_get_matrix(self._h, int(i), int(which), _dp(out))
        if rc < 0:
            raise RuntimeError("get_matrix failed: " + _err(self._lib))
        return out

    def fragments(self, rcut=3.0, at1=1, at2=0):
        """Fragment numbers of every atom (1-based, per molecule) and fragment
        counts at the current coordinates, as fragment_structure
        (src/fragments.f90:93-182); md.f90:450 uses rcut 3.0, at1 1, at2 0."""
        frag = np.zeros(self.natom, dtype=np.int32)
        nfrag = np.zeros(self.nmol, dtype=np.int32)
        self._check(self._lib.qcx_batch_fragments(self._h, float(rcut), int(at1), int(at2), _ip(frag), _ip(nfrag)),
                    "fragments")
        return frag, nfrag

    def set_md_rules(self, nfragexit=2, more=250, max_steps=10000):
        """Run the MD bookkeeping and exit rules of an electron-impact
        fragmentation run (src/md.f90:285-682) on the device after every step;
        call after egrad() of the start geometry."""
        self._check(self._lib.qcx_batch_set_md_rules(self._h, int(nfragexit), int(more), int(max_steps)),
                    "set_md_rules")

    def set_md_heating(self, eimp, tadd, tstep, velof=None):
        """Heating of the first steps (impactscale, src/impact.f90:12-55):
        eimp[nmol] (Eh), tadd[nmol] (atomic time units), velof[natom] or None;
        call before set_md_rules."""
        eimp = np.ascontiguousarray(eimp, dtype=np.float64)
        tadd = np.ascontiguousarray(tadd, dtype=np.float64)
        vf = None if velof is None else np.ascontiguousarray(velof, dtype=np.float64)
        self._check(self._lib.qcx_batch_set_md_heating(self._h, _dp(eimp), _dp(tadd), _dp(vf), float(tstep)),
                    "set_md_heating")

    def set_scc_budget(self, iters):
        """SCC iterations per step for the batch's largest molecule (0: none);
        a molecule whose SCC needs more continues it in the next step without
        moving (status STATUS_SCC_PENDING)."""
        self._check(self._lib.qcx_batch_set_scc_budget(self._h, int(iters)), "set_scc_budget")

    def set_keep_mo(self, on=True):
        """Keep the orbitals of the FP64 SCC for mo_populations (set before egrad)."""
        self._check(self._lib.qcx_batch_set_keep_mo(self._h, int(bool(on))), "set_keep_mo")

    def mo_populations(self, i):
        """(emo [nao] in Eh, focc [nao], qmo [nao][nat], ihomo) of molecule i
        after egrad with set_keep_mo (FP64 precision)."""
        nat = int(self.nat[i])
        from .basis import nao_of
        n = nao_of(self.Z[self.offsets[i]:self.offsets[i] + nat])
        emo, focc, qmo = np.zeros(n), np.zeros(n), np.zeros((n, nat))
        ih = np.zeros(1, dtype=np.int32)
        rc = self._lib.qcx_batch_mo_populations(self._h, int(i), _dp(emo), _dp(focc), _dp(qmo), _ip(ih))
        if rc < 0:
            raise RuntimeError("mo_populations failed: " + _err(self._lib))
        return emo, focc, qmo, int(ih[0])

    def set_md_etemp(self, ax=0.0, ieetemp=0.0):
        """Per-step electronic temperature of EI runs (setetemp after every step).
        Call after set_md_heating and before the start's egrad."""
        self._check(self._lib.qcx_batch_set_md_etemp(self._h, float(ax), float(ieetemp)), "set_md_etemp")

    def md_etemp(self):
        e = np.zeros(self.nmol)
        self._check(self._lib.qcx_batch_get_md_etemp(self._h, _dp(e)), "md_etemp")
        return e

    def set_cid_rules(self, tinit, ntot):
        """Stop rules of the collision MD (src/cid.f90:739-1052) on the device;
        every molecule is the ion followed by one gas atom. Call after egrad()."""
        self._check(self._lib.qcx_batch_set_cid_rules(self._h, float(tinit), int(ntot)), "set_cid_rules")

    def cid_avg_xyz(self):
        """The collision loop's averaged structures [natom][3] (src/cid.f90:1095-1101)."""
        a = np.zeros((self.natom, 3))
        self._check(self._lib.qcx_batch_get_cid_avg_xyz(self._h, _dp(a)), "cid_avg_xyz")
        return a

    def cid_state(self):
        n = self.nmol
        i32 = lambda: np.zeros(n, dtype=np.int32)
        v = {k: i32() for k in ("nstep", "nfrag", "collided", "fragmented", "total_steps", "done", "failed")}
        avg_t, ecom = np.zeros(n), np.zeros(n)
        self._check(self._lib.qcx_batch_get_cid_state(self._h, _ip(v["nstep"]), _ip(v["nfrag"]), _ip(v["collided"]),
                                                      _ip(v["fragmented"]), _ip(v["total_steps"]), _ip(v["done"]),
                                                      _ip(v["failed"]), _dp(avg_t), _dp(ecom)), "cid_state")
        v["avg_temp"], v["ecom_ev"] = avg_t, ecom
        return v

    def md_avg_xyz(self):
        """Averaged structure (src/md.f90:352-362, 695) of every trajectory, [natom][3]."""
        out = np.zeros((self.natom, 3))
        self._check(self._lib.qcx_batch_get_md_avg_xyz(self._h, _dp(out)), "md_avg_xyz")
        return out

    def md_state(self):
        n = self.nmol
        i32 = lambda: np.zeros(n, dtype=np.int32)
        nstep, nfrag, fragstate, mdok, done = i32(), i32(), i32(), i32(), i32()
        tav, eerror, fragT = np.zeros(n), np.zeros(n), np.zeros((n, 10))
        self._check(self._lib.qcx_batch_get_md_state(self._h, _ip(nstep), _ip(nfrag), _ip(fragstate), _ip(mdok),
                                                     _ip(done), _dp(tav), _dp(eerror), _dp(fragT)), "md_state")
        return {"nstep": nstep, "nfrag": nfrag, "fragstate": fragstate, "mdok": mdok, "done": done, "tav": tav,
                "eerror": eerror, "fragT": fragT}

    def progress(self):
        active = np.zeros(self.nmol, dtype=np.int32)
        steps = np.zeros(self.nmol, dtype=np.int64)
        self._check(self._lib.qcx_batch_get_progress(self._h, _ip(active),
                                                     steps.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))),
                    "progress")
        return active, steps

    def stream(self):
        return int(self._lib.qcx_batch_stream(self._h))

    def profile_egrad(self):
        ms = np.zeros(6, dtype=np.float32)
        self._check(self._lib.qcx_batch_profile_egrad(self._h, ms.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
                    "profile_egrad")
        return dict(zip(["cn", "integrals", "scc", "zero_grad", "grad_pairs", "grad_atoms"], ms.tolist()))

    def set_timing(self, on=True):
        """Record timing marks inside the captured step graph (per molecule group:
        integrals start, SCC start, SCC end, gradient end)."""
        self._check(self._lib.qcx_batch_set_timing(self._h, int(bool(on))), "set_timing")

    def timing(self):
        """Marks of the last replayed step in ms from its start: dict with
        'step' (total), 'scc_span' (first SCC start to last SCC end over the
        groups), 'scc_sum' (sum of the groups' SCC durations) and the raw marks
        [G][4]."""
        buf = np.zeros(2 + 4 * 64, dtype=np.float32)
        g = self._lib.qcx_batch_get_timing(self._h, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(buf))
        if g < 0:
            raise RuntimeError("get_timing failed: " + _err(self._lib))
        marks = buf[1:1 + 4 * g].reshape(g, 4).astype(np.float64)
        return {"step": float(buf[1 + 4 * g]), "scc_span": float(marks[:, 2].max() - marks[:, 1].min()),
                "scc_sum": float(np.sum(marks[:, 2] - marks[:, 1])), "marks": marks}

    def sizes(self):
        nao = np.zeros(self.nmol, dtype=np.int32)
        nat = np.zeros(self.nmol, dtype=np.int32)
        self._check(self._lib.qcx_batch_get_sizes(self._h, _ip(nao), _ip(nat)), "sizes")
        return nao, nat

    def set_state_ptr(self, xyz_ptr=None, vel_ptr=None):
        """set_state from raw host pointers (e.g. pinned buffers)."""
        c = lambda p: None if p is None else ctypes.cast(p, ctypes.POINTER(ctypes.c_double))
        self._check(self._lib.qcx_batch_set_state(self._h, c(xyz_ptr), c(vel_ptr), None), "set_state")

    def load_state_ptr(self, xyz_ptr=None, vel_ptr=None):
        """qcx_batch_load_state from raw host pointers: new coordinates and
        velocities for the running trajectories (stopped ones stay stopped)."""
        c = lambda p: None if p is None else ctypes.cast(p, ctypes.POINTER(ctypes.c_double))
        self._check(self._lib.qcx_batch_load_state(self._h, c(xyz_ptr), c(vel_ptr)), "load_state")

    def get_ptr(self, xyz_ptr=None, vel_ptr=None, energy_ptr=None):
        """get into raw host pointers (e.g. pinned buffers)."""
        c = lambda p: None if p is None else ctypes.cast(p, ctypes.POINTER(ctypes.c_double))
        self._check(self._lib.qcx_batch_get(self._h, c(xyz_ptr), c(vel_ptr), None, c(energy_ptr), None, None,
                                            None, None), "get")

    def kernel_launches(self):
        return int(self._lib.qcx_batch_kernel_launches(self._h))

    def split(self, arr):
        return [arr[self.offsets[i]:self.offsets[i + 1]] for i in range(self.nmol)]

    def close(self):
        if getattr(self, "_h", None):
            self._lib.qcx_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
