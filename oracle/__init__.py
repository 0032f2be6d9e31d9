"""ctypes binding of the CPU FP64 oracle -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py``, where it is the checker (or the timed CPU baseline), never
the thing measured as the product. Parity with tblite is unpinned: see
``qcx_oracle.h``.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqcxoracle.so")


def build(force=False):
    src = os.path.join(HERE, "qcx_oracle.c")
    deps = [src, os.path.join(HERE, "qcx_oracle.h"),
            os.path.join(HERE, "..", "qcxms_gb300", "csrc", "qcx_params.h"),
            os.path.join(HERE, "..", "qcxms_gb300", "csrc", "qcx_consts.h"),
            os.path.join(HERE, "..", "qcxms_gb300", "csrc", "qcx_d4ref.h")]
    if not force and os.path.exists(LIB_PATH) and \
            os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(d) for d in deps):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp", "-o", LIB_PATH, src, "-lm"]
    subprocess.check_call(cmd)
    return LIB_PATH


class Opts(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int), ("econv", ctypes.c_double),
                ("pconv", ctypes.c_double), ("broyden_alpha", ctypes.c_double)]


class Info(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("e_band", "e_ies", "e_3", "e_aes", "e_axc", "e_disp", "e_atm", "e_rep", "e_ts", "e_total")] + \
               [("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("nao", ctypes.c_int),
                ("nsh", ctypes.c_int), ("nel", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.qcxo_egrad.restype = ctypes.c_int
        _lib.qcxo_nao.restype = ctypes.c_int
        _lib.qcxo_nsh.restype = ctypes.c_int
        _lib.qcxo_gnorm.restype = ctypes.c_double
        _lib.qcxo_getspin.restype = ctypes.c_int
        _lib.qcxo_checkqc.restype = ctypes.c_int
        _lib.qcxo_fragments.restype = ctypes.c_int
        _lib.qcxo_md_batch.restype = ctypes.c_int
        _lib.qcxo_egrad_batch.restype = ctypes.c_int
        _lib.qcxo_eself.restype = ctypes.c_double
        _lib.qcxo_d4_c6ref.restype = ctypes.c_double
        _lib.qcxo_nel.restype = ctypes.c_int
    return _lib


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


def default_opts(**kw):
    o = Opts()
    lib().qcxo_default_opts(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def nao(Z):
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    return lib().qcxo_nao(len(Z), _p(Z, ctypes.c_int))


def nsh(Z):
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    return lib().qcxo_nsh(len(Z), _p(Z, ctypes.c_int))


def egrad(Z, xyz, charge=0, kT=300.0 * 3.166808578545117e-06, opts=None):
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    nat = len(Z)
    e = ctypes.c_double()
    g = np.zeros((nat, 3))
    q = np.zeros(nat)
    info = Info()
    o = opts if opts is not None else default_opts()
    rc = lib().qcxo_egrad(nat, _p(Z, ctypes.c_int), _p(xyz), ctypes.c_double(charge), ctypes.c_double(kT),
                          ctypes.byref(o), ctypes.byref(e), _p(g), _p(q), ctypes.byref(info))
    return rc, e.value, g, q, info.as_dict()


def integrals(Z, xyz):
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n = nao(Z)
    S = np.zeros((n, n)); H0 = np.zeros((n, n))
    Dm = np.zeros((3, n, n)); Qm = np.zeros((6, n, n))
    cn = np.zeros(len(Z)); cnd = np.zeros(len(Z))
    rc = lib().qcxo_integrals(len(Z), _p(Z, ctypes.c_int), _p(xyz), _p(S), _p(H0), _p(Dm), _p(Qm), _p(cn), _p(cnd))
    assert rc == 0
    return S, H0, Dm, Qm, cn, cnd


def scc(Z, xyz, charge=0, kT=300.0 * 3.166808578545117e-06, opts=None):
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n, ns, nat = nao(Z), nsh(Z), len(Z)
    P = np.zeros((n, n)); qsh = np.zeros(ns); dp = np.zeros((nat, 3)); qp = np.zeros((nat, 6))
    eps = np.zeros(n); focc = np.zeros(n)
    info = Info()
    o = opts if opts is not None else default_opts()
    rc = lib().qcxo_scc(nat, _p(Z, ctypes.c_int), _p(xyz), ctypes.c_double(charge), ctypes.c_double(kT),
                        ctypes.byref(o), _p(P), _p(qsh), _p(dp), _p(qp), _p(eps), _p(focc), ctypes.byref(info))
    assert rc == 0
    return P, qsh, dp, qp, eps, focc, info.as_dict()


def mo_spectrum(Z, xyz, charge=0, kT=300.0 * 3.166808578545117e-06, opts=None):
    """write_qmo's quantities (src/mo_energ.f90:7-80) of the converged SCC:
    returns (rc, emo [nao] in Eh, focc [nao], qmo [nao][nat], ihomo, info)."""
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    n, nat = nao(Z), len(Z)
    emo = np.zeros(n); focc = np.zeros(n); qmo = np.zeros((n, nat))
    ih = ctypes.c_int()
    info = Info()
    o = opts if opts is not None else default_opts()
    rc = lib().qcxo_mo_spectrum(nat, _p(Z, ctypes.c_int), _p(xyz), ctypes.c_double(charge), ctypes.c_double(kT),
                                ctypes.byref(o), _p(emo), _p(focc), _p(qmo), ctypes.byref(ih), ctypes.byref(info))
    return rc, emo, focc, qmo, ih.value, info.as_dict()


def syev(A):
    A = np.array(A, dtype=np.float64, order="C")
    n = A.shape[0]
    w = np.zeros(n); V = np.zeros((n, n))
    rc = lib().qcxo_syev(n, _p(A), _p(w), _p(V))
    return rc, w, V


def leapfrog(grad, mass, tstep, xyz, vel):
    grad = np.ascontiguousarray(grad, dtype=np.float64)
    mass = np.ascontiguousarray(mass, dtype=np.float64)
    xyz = np.array(xyz, dtype=np.float64, order="C")
    vel = np.array(vel, dtype=np.float64, order="C")
    ke = ctypes.c_double()
    lib().qcxo_leapfrog(len(mass), _p(grad), _p(mass), ctypes.c_double(tstep), _p(xyz), _p(vel), ctypes.byref(ke))
    return xyz, vel, ke.value


def getspin(Z, charge):
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    return lib().qcxo_getspin(len(Z), _p(Z, ctypes.c_int), int(charge))


AUTOEV = 27.21138505  # src/xtb_mctc_convert.f90:27
AUTOKCAL = 627.50947428  # src/xtb_mctc_convert.f90:30
KB = 3.166808578545117e-06  # src/xtb_mctc_constants.f90:35


def eself(Z):
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    return lib().qcxo_eself(len(Z), _p(Z, ctypes.c_int))


def nel(Z, charge):
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    return lib().qcxo_nel(len(Z), _p(Z, ctypes.c_int), int(charge))


def fragment_ips(Z, xyz, frag, mchrg=1, etemp=300.0, opts=None, iterations=False):
    """IPs/EAs of the fragments of one structure, restating the GFN2 path of
    analyse (src/analyse.f90:13-467) with eqm (src/iniqm.f90:241-427).

    Returns (fragip (nfrag, |mchrg|) in eV, energies (nfrag, |mchrg|+1) in Eh,
    ipok), plus the largest SCC iteration count of its single points when
    ``iterations`` is set."""
    Z = np.asarray(Z, dtype=np.int32)
    xyz = np.asarray(xyz, dtype=np.float64).reshape(len(Z), 3)
    frag = np.asarray(frag)
    nfrag = int(frag.max())
    nch = abs(mchrg)
    fragip = np.zeros((nfrag, nch))
    E = np.zeros((nfrag, nch + 1))
    ipok = True
    maxit = 0
    if nfrag < 2:  # src/analyse.f90:137-142
        return (fragip, E, ipok, maxit) if iterations else (fragip, E, ipok)
    for i in range(nfrag):
        # avg_frag_struc (src/analyse.f90:471-503): atoms of fragment i in their order
        sel = np.nonzero(frag == i + 1)[0]
        Zf, xf = Z[sel], xyz[sel]
        for c in range(nch + 1):
            ch = c if mchrg > 0 else -c
            ne = nel(Zf, ch)
            if ne == 0:
                E[i, c] = eself(Zf)
            elif ne > 0:
                rc, e, g, q, info = egrad(Zf, xf, ch, kT=etemp * KB, opts=opts)
                E[i, c] = e if rc == 0 else 0.0
                maxit = max(maxit, info["iterations"])
            if abs(E[i, c]) < 1e-10:  # src/iniqm.f90:415-421
                ipok = False
        for c in range(1, nch + 1):
            if E[i, c] != 0 and E[i, 0] != 0:  # src/analyse.f90:367-403
                ip = (E[i, c] - E[i, 0]) * AUTOEV
                fragip[i, c - 1] = ip
                if mchrg < 0:
                    bad = ip > 40.0 or ip < -35.0
                elif mchrg == 1:
                    bad = ip < 0.0 or ip > 50.0
                else:
                    bad = ip < 0.0 or ip > 100.0
                if bad:
                    ipok = False
    return (fragip, E, ipok, maxit) if iterations else (fragip, E, ipok)


def boltz(units, temp, ip):
    """boltz (src/utility.f90:469-498), loop for loop."""
    const = AUTOKCAL if units == 1 else AUTOEV
    f = temp * KB * const
    nfrag, mchrg = ip.shape
    esum = 0.0
    for i in range(nfrag):
        for j in range(mchrg):
            esum = esum + np.exp(-ip[i, j] / f)
    out = np.zeros_like(ip)
    for i in range(nfrag):
        for j in range(mchrg):
            out[i, j] = np.exp(-ip[i, j] / f) / esum
    return out


FSTOAU = 41.3413733365614  # src/xtb_mctc_convert.f90:54


def _temp(e, n):
    """e / (0.5*3*n*kB) with 0.5*3*n in default (single) real (src/md.f90:289, 736)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.float64(e) / (float(np.float32(1.5) * np.float32(n)) * KB))


def md_rules_top(s, epot, ekin, nuc, xyz=None):
    """Top of the MD loop (src/md.f90:286-362), it > 0, isec = 1; with xyz the
    running coordinate sum of the averaged structure (window of 50 steps)."""
    s["nstep"] += 1
    t = _temp(ekin, nuc)
    s["tav"] = s["tav"] + t
    s["epav"] = s["epav"] + epot
    s["ekav"] = s["ekav"] + ekin
    if s["nstep"] > s["nadd"]:
        s["edum"] = (s["edum"] + epot) + ekin
        eav = s["edum"] / float(np.float32(s["nstep"] - s["nadd"]))
    else:
        eav = epot + ekin
    s["eerror"] = (eav - epot) - ekin
    if s["nfrag"] == 1:
        s["fragT"][0] = s["tav"] / s["nstep"]
    if epot == 0 or abs(s["eerror"]) > float(np.float32(0.1)):
        s["mdok"] = 1 if 1 < s["nfrag"] <= 4 else 0
        s["done"] = 1
        return True
    if s["kdump"] > 50 - 1:
        s["kdump"] = 0
        s["avxyz"] = None
    if xyz is not None:
        if s["avxyz"] is None:
            s["avxyz"] = [[0.0, 0.0, 0.0] for _ in range(nuc)]
        for i in range(nuc):
            for d in range(3):
                s["avxyz"][i][d] = s["avxyz"][i][d] + xyz[i][d]
    return False


def md_avg_xyz(s):
    """axyz = avxyz / kdump (src/md.f90:695)."""
    return [[c / s["kdump"] for c in row] for row in s["avxyz"]]


def _ekinet(vel, mass, velof=None, scal=0.0):
    """ekinet (src/mdinit.f90:57-76) of vel * (1 + velof * scal)."""
    ek = 0.0
    for i in range(len(mass)):
        f = 1.0 + (1.0 if velof is None else velof[i]) * scal
        x, y, z = vel[i][0] * f, vel[i][1] * f, vel[i][2] * f
        ek = ek + mass[i] * ((x * x + y * y) + z * z)
    return ek * 0.5


def impactscale(vel, mass, velof, eimp, ff, e0):
    """impactscale (src/impact.f90:12-55); scales vel in place, False after
    20000 increments."""
    esoll = eimp * ff + e0
    scal, k = 0.0, 0
    while True:
        k += 1
        e = _ekinet(vel, mass, velof, scal)
        scal = scal + float(np.float32(0.0002))
        if not (esoll - e > float(np.float32(0.001)) and k < 20000):
            break
    for i in range(len(mass)):
        f = 1.0 + (1.0 if velof is None else velof[i]) * scal
        for d in range(3):
            vel[i][d] = vel[i][d] * f
    return k < 20000


def md_heating(eimp, tadd, tstep):
    """(eimp, fadd, nadd) of src/md.f90:265-266."""
    return eimp, tstep / (tadd + tstep), int((tadd + tstep) / tstep - 1.0)


def setetemp(nfrag, eimp, ax, ieetemp):
    """setetemp (src/utility.f90:69-86): 5000. + 20000.*ax, plus max(eimp, 0)*ieetemp
    while eimp > 0 and nfrag <= 1 (5000. and 20000. are exact single-precision literals)."""
    etemp = 5000.0 + 20000.0 * ax
    if eimp > 0 and nfrag <= 1:
        etemp = etemp + max(eimp, 0.0) * ieetemp
    return etemp


def md_rules_begin(vel, mass, epot, heat=None, xyz=None, etemp=None):
    """State before the loop: ekinet (src/mdinit.f90:57-76) and the first top.
    heat = (eimp, fadd, nadd) of md_heating, or None; etemp = (ax, ieetemp) for the
    per-step electronic temperature, or None."""
    s = {"nstep": 0, "nfrag": 1, "fconst": 0, "morestep": 0, "fragstate": 0, "mdok": 0, "done": 0, "tav": 0.0,
         "epav": 0.0, "ekav": 0.0, "edum": 0.0, "eerror": 0.0, "ttime": 0.0, "dtime": 0.0, "fragT": [0.0] * 10,
         "eimp": 0.0, "fadd": 0.0, "nadd": 0, "heat_failed": 0, "kdump": 50, "avxyz": None, "etemp": -1.0}
    if heat is not None:
        s["eimp"], s["fadd"], s["nadd"] = heat
    if etemp is not None:
        s["etemp"] = setetemp(1, s["eimp"], *etemp)  # src/md.f90:167-168
    ek = _ekinet(vel, mass)
    s["ekinstart"] = ek
    if epot == 0:
        s["done"] = 1  # src/md.f90:185
    else:
        md_rules_top(s, epot, ek, len(mass), xyz)
    return s


def md_rules_step(s, epot, ekin, vel, mass, frag, nfrag, tstep, nfragexit, more, max_steps, velof=None, xyz=None,
                  etemp=None):
    """Rest of one loop iteration after leapfrog + egrad (src/md.f90:426-679,
    electron-impact branch), then the next top. epot = 0 for a failed call.
    vel (the velocities after leapfrog) is scaled in place while heating.
    etemp = (ax, ieetemp): s["etemp"] becomes the next evaluation's electronic
    temperature (src/md.f90:443-446)."""
    if s["done"]:
        return s
    s["ttime"] = s["ttime"] + tstep / FSTOAU
    s["kdump"] += 1  # src/md.f90:400
    if s["nfrag"] == 1:
        s["morestep"] = 0
    if s["nfrag"] > 1 and s["dtime"] < 1.0e-6:
        s["dtime"] = s["ttime"] / 1000.0
    if s["nstep"] <= s["nadd"] and s["nfrag"] == 1:  # src/md.f90:439-441
        if not impactscale(vel, mass, velof, s["eimp"], s["fadd"] * s["nstep"], s["ekinstart"]):
            s["heat_failed"], s["done"] = 1, 1
            return s
    if etemp is not None:  # src/md.f90:443-446, with the previous step's fragment count
        dum = s["eimp"] - s["eimp"] * float(np.float32(s["nstep"])) / float(np.float32(s["nadd"])) \
            if s["nadd"] != 0 else float("nan")
        s["etemp"] = setetemp(s["nfrag"], dum, *etemp)
    s["nfrag"] = nfrag
    if nfrag > 1:  # intenergy, src/md.f90:715-741
        eint, cnt = [0.0] * 10, [0] * 10
        for i in range(len(mass)):
            j = frag[i] - 1
            if j >= 10:
                continue
            v = vel[i]
            eint[j] = eint[j] + (0.5 * mass[i]) * ((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])
            cnt[j] += 1
        for j in range(min(nfrag, 10)):
            s["fragT"][j] = _temp(eint[j], cnt[j])
    stop = False
    if nfrag > 6:
        stop = True
    elif nfrag > nfragexit:
        s["fragstate"], s["mdok"], stop = 1, 1, True
    else:
        s["fconst"] = s["fconst"] + 1 if nfrag >= 2 else 0
        if s["fconst"] > 1000:
            s["fragstate"], s["mdok"], stop = 2, 1, True
        elif nfrag >= nfragexit:
            s["morestep"] += 1
            if s["morestep"] > more:
                s["fragstate"], s["mdok"], stop = 1, 1, True
    if not stop and s["nstep"] >= max_steps:
        s["fragstate"], s["mdok"], stop = 1, 1, True
    if stop:
        s["done"] = 1
    else:
        md_rules_top(s, epot, ekin, len(mass), xyz)
    return s


def _com(xyz, mass, nuc):
    """center_of_mass (src/utility.f90:541-562) of the first nuc atoms."""
    cm, tm = [0.0, 0.0, 0.0], 0.0
    for i in range(nuc):
        for d in range(3):
            cm[d] = cm[d] + mass[i] * xyz[i][d]
        tm = tm + mass[i]
    return [c / tm for c in cm]


def _norm3(x, y, z):
    return float(np.sqrt((x * x + y * y) + z * z))


def cid_rules_begin(xyz, mass, ntot):
    """State before the collision loop (src/cid.f90:715-724); the last atom is the gas atom."""
    nuc = len(mass) - 1
    s = {"nstep": 0, "m": 0, "step_counter": 0, "collided": 0, "fragmented": 0, "total_steps": ntot, "nfrag": 1,
         "done": 0, "failed": 0, "distance_dump": 0, "ttime": 0.0, "tav": 0.0, "avgT": 0.0, "new_temp": 0.0,
         "ecom": 0.0}
    sm = 0.0
    for i in range(nuc):
        sm = sm + mass[i]
    s["summass"] = sm
    cm = _com(xyz, mass, nuc)
    s["old_cm"] = cm
    g = xyz[nuc]
    d0 = _norm3(g[0] - cm[0], g[1] - cm[1], g[2] - cm[2])
    s["lowest"] = s["highest"] = d0
    # averaged structures: avxyz = avxyz2 = 0 (src/cid.f90:244-245), xyzavg_dump = 0
    # (:715), check_fragmented = 1 (:265), count_average .false. (:147); save_natf
    # has no initial value in the reference (0 here)
    s["avxyz"] = np.zeros((nuc, 3))
    s["avxyz2"] = np.zeros((nuc, 3))
    s["store"] = np.zeros((nuc, 3))
    s["xyzavg_dump"], s["cnt"], s["count_average"], s["check_fragmented"] = 0, 0, 0, 1
    s["save_natf"] = [0] * 10
    return s


def _cid_average(s, xyz, nfrag, frag):
    """src/cid.f90:802-909: the averaged structures after the fragment count."""
    nuc = s["avxyz"].shape[0]
    x = np.asarray(xyz, dtype=np.float64)[:nuc]
    s["avxyz"] = s["avxyz"] + x
    if nfrag > s["check_fragmented"]:
        s["count_average"] = 1
        s["check_fragmented"] = nfrag
    if nfrag < s["check_fragmented"] and s["count_average"]:
        s["cnt"] = 0
        s["avxyz2"] = np.zeros((nuc, 3))
        s["store"] = np.zeros((nuc, 3))
        s["count_average"] = 0
        s["check_fragmented"] = 1
    if s["count_average"]:
        s["cnt"] += 1
        s["avxyz2"] = s["avxyz2"] + x
        s["store"] = s["avxyz2"] / s["cnt"]
        # avg_frag_struc (src/analyse.f90:452-502): atoms per fragment
        natf = [0] * 10
        for lab in list(frag)[:nuc]:
            if 1 <= lab <= 10:
                natf[lab - 1] += 1
        for k in range(min(nfrag, 10)):
            if s["cnt"] == 1:
                s["save_natf"][k] = natf[k]
            if natf[k] != s["save_natf"][k]:
                s["cnt"] = 0
                s["store"] = np.zeros((nuc, 3))
                s["avxyz2"] = np.zeros((nuc, 3))
                break
        if s["cnt"] == 50:
            s["store"] = s["avxyz2"] / s["cnt"]
            s["avxyz2"] = np.zeros((nuc, 3))
            s["cnt"] = 0
            s["count_average"] = 0


def cid_avg_xyz(s):
    """The averaged structure the collision loop returns (src/cid.f90:1095-1101)."""
    if s["check_fragmented"] > 1:
        return s["store"].copy()
    return s["avxyz"] / s["xyzavg_dump"]


def cid_rules_step(s, failed, xyz, vel, mass, nfrag, tstep, tinit, frag=None):
    """One step of the collision loop after leapfrog + egrad (src/cid.f90:739-1036).
    frag: the ion's fragment numbers (for the averaged structures; every atom in
    fragment 1 when not given)."""
    if s["done"]:
        return s
    autofs = 1.0 / FSTOAU
    mstoau = 1.0 / 2.18769126364e6
    nuc = len(mass) - 1
    s["nstep"] += 1
    if s["xyzavg_dump"] == 50:  # src/cid.f90:743-746
        s["xyzavg_dump"] = 0
        s["avxyz"] = np.zeros((nuc, 3))
    s["ttime"] = s["ttime"] + tstep * autofs
    s["distance_dump"] += 1
    s["xyzavg_dump"] += 1
    if failed:
        s["done"], s["failed"] = 1, 1
        return s
    cm = _com(xyz, mass, nuc)
    oc = s["old_cm"]
    cm_out = _norm3(cm[0] - oc[0], cm[1] - oc[1], cm[2] - oc[2])
    s["old_cm"] = cm
    new_velo = (cm_out / tstep) / mstoau if s["nstep"] != 1 else 0.0
    ek = 0.0
    for i in range(nuc):
        v = vel[i]
        ek = ek + mass[i] * ((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2])
    ek = ek * 0.5
    x = new_velo * mstoau
    e_velo = (0.5 * s["summass"]) * (x * x)
    ekd = ek - e_velo
    s["new_temp"] = (2.0 * ekd) / ((3.0 * KB) * float(nuc))
    if s["nstep"] == 1:
        s["new_temp"] = tinit
    s["tav"] = s["tav"] + s["new_temp"]
    s["m"] += 1
    s["avgT"] = s["tav"] / s["m"]
    mgas = mass[nuc]
    s["ecom"] = ((mgas / (mgas + s["summass"])) * e_velo) * AUTOEV
    s["nfrag"] = nfrag
    _cid_average(s, xyz, nfrag, frag if frag is not None else [1] * nuc)
    if s["distance_dump"] == 10:
        s["distance_dump"] = 0
        g = xyz[nuc]
        dist = _norm3(g[0] - cm[0], g[1] - cm[1], g[2] - cm[2])
        if dist > s["highest"]:
            s["highest"] = dist
        if dist < s["lowest"]:
            s["lowest"] = dist
        s["step_counter"] = s["step_counter"] + 1 if s["lowest"] < dist else 0
        if s["step_counter"] == 5:
            s["collided"] = 1
            t = 800.0 * ((2.0 * tstep) * autofs)
            q = float(np.floor(t))  # nint: half away from zero (t > 0)
            s["total_steps"] = s["nstep"] + int(q) + (1 if t - q >= 0.5 else 0)
            s["tav"], s["m"] = 0.0, 0
    if nfrag > 1 and s["collided"] and not s["fragmented"]:
        add = (nuc // 10) * 1000 if nuc >= 40 else ((nuc // 10) * 500 if nuc > 10 else 0)
        s["total_steps"] = s["nstep"] + add
        s["fragmented"] = 1
    if s["nstep"] >= s["total_steps"]:
        s["done"] = 1
    return s


def d4_c6ref(za, i, zb, j):
    """C6 of D4 reference pair (za, i; zb, j), 0-based reference indices."""
    return lib().qcxo_d4_c6ref(int(za), int(i), int(zb), int(j))


def d4_c6(Z, xyz, q=None):
    """Molecular D4 C6 [nat][nat] at the covalent CNs and charges q (zero if None)."""
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(len(Z), 3)
    c6 = np.zeros((len(Z), len(Z)))
    qq = None if q is None else np.ascontiguousarray(q, dtype=np.float64)
    lib().qcxo_d4_c6(len(Z), _p(Z, ctypes.c_int), _p(xyz), None if qq is None else _p(qq), _p(c6))
    return c6


def gnorm(grad):
    grad = np.ascontiguousarray(grad, dtype=np.float64)
    return lib().qcxo_gnorm(grad.shape[0], _p(grad))


def checkqc(e, grad, qat, charge):
    grad = np.ascontiguousarray(grad, dtype=np.float64)
    qat = np.ascontiguousarray(qat, dtype=np.float64)
    ee = ctypes.c_double(e)
    ok = lib().qcxo_checkqc(grad.shape[0], ctypes.byref(ee), _p(grad), _p(qat), int(charge))
    return bool(ok), ee.value


def fragments(Z, xyz, rcut=3.0, at1=1, at2=0):
    """Fragment numbers (1-based) of every atom and the fragment count, as
    fragment_structure (src/fragments.f90:93-182)."""
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(len(Z), 3)
    frag = np.zeros(len(Z), dtype=np.int32)
    nf = lib().qcxo_fragments(len(Z), _p(Z, ctypes.c_int), _p(xyz), ctypes.c_double(rcut), int(at1), int(at2),
                              _p(frag, ctypes.c_int))
    return frag, nf


def egrad_batch(mols, kT, opts=None, nthreads=0):
    """Energies, gradients and charges of many structures (dicts with Z, xyz,
    charge), OpenMP over structures. Returns (rc[n], energy[n], grads, qats)."""
    off = np.zeros(len(mols) + 1, dtype=np.int32)
    for i, m in enumerate(mols):
        off[i + 1] = off[i] + len(m["Z"])
    Z = np.ascontiguousarray(np.concatenate([m["Z"] for m in mols]), dtype=np.int32)
    xyz = np.ascontiguousarray(np.concatenate([np.asarray(m["xyz"]).reshape(-1, 3) for m in mols]), dtype=np.float64)
    charge = np.array([m["charge"] for m in mols], dtype=np.float64)
    kTa = np.full(len(mols), kT, dtype=np.float64)
    e = np.zeros(len(mols))
    g = np.zeros((off[-1], 3))
    q = np.zeros(off[-1])
    rc = np.zeros(len(mols), dtype=np.int32)
    o = opts if opts is not None else default_opts()
    lib().qcxo_egrad_batch(len(mols), _p(off, ctypes.c_int), _p(Z, ctypes.c_int), _p(xyz), _p(charge), _p(kTa),
                           ctypes.byref(o), int(nthreads), _p(e), _p(g), _p(q), _p(rc, ctypes.c_int))
    return rc, e, [g[off[i]:off[i + 1]] for i in range(len(mols))], [q[off[i]:off[i + 1]] for i in range(len(mols))]


def md_batch(mols, nsteps, tstep, grad0, kT, opts=None, nthreads=0, active=None, steps_done=None, busy_s=None):
    """CPU MD over a list of molecules (dicts with Z, xyz, vel, mass, charge).
    With ``active`` (int32 array, updated in place) failed trajectories stop;
    ``steps_done`` (int32 array) receives the accepted steps per trajectory."""
    off = np.zeros(len(mols) + 1, dtype=np.int32)
    for i, m in enumerate(mols):
        off[i + 1] = off[i] + len(m["Z"])
    Z = np.ascontiguousarray(np.concatenate([m["Z"] for m in mols]), dtype=np.int32)
    xyz = np.ascontiguousarray(np.concatenate([m["xyz"] for m in mols]), dtype=np.float64)
    vel = np.ascontiguousarray(np.concatenate([m["vel"] for m in mols]), dtype=np.float64)
    mass = np.ascontiguousarray(np.concatenate([m["mass"] for m in mols]), dtype=np.float64)
    grad = np.ascontiguousarray(np.concatenate(grad0), dtype=np.float64)
    charge = np.array([m["charge"] for m in mols], dtype=np.float64)
    kTa = np.full(len(mols), kT, dtype=np.float64)
    epot = np.zeros(len(mols))
    iters = np.zeros(len(mols), dtype=np.int32)
    o = opts if opts is not None else default_opts()
    fails = lib().qcxo_md_batch(len(mols), _p(off, ctypes.c_int), _p(Z, ctypes.c_int), _p(xyz), _p(vel), _p(mass),
                                _p(grad), _p(epot), _p(charge), _p(kTa), int(nsteps), ctypes.c_double(tstep),
                                ctypes.byref(o), int(nthreads), _p(iters, ctypes.c_int),
                                None if active is None else _p(active, ctypes.c_int),
                                None if steps_done is None else _p(steps_done, ctypes.c_int),
                                None if busy_s is None else _p(busy_s))
    return fails, xyz, vel, grad, epot, iters
