"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm import this module; the product library never does.  The C restatement
it wraps (oracle/cans_oracle.c) follows the reference's CPU path file by file
(citations in that file) and is pinned by the lid-driven-cavity golden vector
of the reference's own regression suite.

Arrays are numpy float64 in Fortran order; haloed fields have shape
(n1+2, n2+2, n3+2) and 1D grid arrays shape (n3+2,), index 0..n3+1.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

HALO_LOWER, HALO_NONE, HALO_UPPER, HALO_BOTH = -1, 0, 1, 2
R2HC, HC2R, REDFT00, REDFT01, REDFT10, REDFT11, RODFT00, RODFT01, RODFT10, RODFT11 = 0, 1, 3, 4, 5, 6, 7, 8, 9, 10

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        _setup(_lib)
    return _lib


def _setup(L):
    L.orc_initgrid.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, _D, _D, _D, _D]
    L.orc_eigenvalues.argtypes = [C.c_int, C.c_char_p, C.c_char, _D]
    L.orc_tridmatrix.argtypes = [C.c_char_p, C.c_int, _D, _D, C.c_char, _D, _D, _D]
    L.orc_initsolver.argtypes = [_I, _D, _D, _D, C.c_char_p, _D, C.c_char_p, _D, _D, _D, _D, _D, _D]
    L.orc_r2r.argtypes = [C.c_int, C.c_int, C.c_long, C.c_long, C.c_long, _D]
    L.orc_r2r_dir.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _D]
    L.orc_gaussel.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _D, _D, _D, C.c_int, C.c_double, _D, _D]
    L.orc_solver.argtypes = [_I, C.c_double, _D, _D, _D, _D, C.c_char_p, C.c_char_p, _D]
    L.orc_solve_helmholtz.argtypes = [_I, C.c_double, C.c_double, _D, _D, _D, _D, _D, _I, C.c_char_p,
                                      C.c_char_p, _D]
    L.orc_fillps.argtypes = [_I, _D, _D, C.c_double, _D, _D, _D, _D]
    L.orc_correc.argtypes = [_I, _D, _D, C.c_double, _D, _D, _D, _D]
    L.orc_updatep.argtypes = [_I, _D, _D, _D, C.c_double, C.c_int, _D, _D]
    L.orc_mom_xyz_ad.argtypes = [_I, C.c_double, C.c_double, _D, _D, C.c_double, _D, _D, _D, _D, _D, _D,
                                 _D, _D, _D, C.c_int]
    L.orc_bulk_mean.argtypes = [_I, _D, _D]
    L.orc_bulk_mean.restype = C.c_double
    L.orc_rk.argtypes = [_D, _I, _D, _D, _D, _D, _D, C.c_double, C.c_double, _D, _I, _D, _D, C.c_int,
                         _D, _D, _D, _D, _D, _D, _D, _D]
    L.orc_rk_buoy.argtypes = [_D, _I, _D, _D, _D, _D, _D, C.c_double, C.c_double, _D, _I, _D, _D, C.c_int,
                              _D, C.c_double, _D, _D, _D, _D, _D, _D, _D, _D, _D]
    L.orc_rk_scal.argtypes = [_D, _I, _D, _D, _D, _D, C.c_double, C.c_double, _D, _D, _D, C.c_int, C.c_double,
                              C.c_double, C.c_int, _D, _D, _D]
    L.orc_rk_scal.restype = C.c_double
    L.orc_bulk_forcing_s.argtypes = [_I, C.c_int, C.c_double, _D]
    L.orc_bounduvw.argtypes = [C.c_char_p, _I, _D, _I, _D, _D, _D, _D, _D, _D, C.c_int, C.c_int, C.c_int]
    L.orc_boundp.argtypes = [C.c_char_p, _I, _D, _I, _D, _D, _D, C.c_int]
    L.orc_updt_rhs_b.argtypes = [C.c_char_p, C.c_char_p, _I, _I, _D, _D, C.c_double, C.c_int]
    L.orc_chkdt.argtypes = [_I, _D, _D, _D, C.c_double, C.c_double, C.c_int, C.c_int, _D, _D, _D]
    L.orc_chkdt.restype = C.c_double
    L.orc_chkdiv.argtypes = [_I, _D, _D, _D, _D, _D, _D, _D, _D]
    L.orc_add_noise.argtypes = [_I, C.c_ulonglong, C.c_double, _D]
    L.orc_poisson_residual_ld.argtypes = [_I, _D, C.c_char_p, _D, _D, _D, _D, _D, _D]
    L.orc_initflow.argtypes = [C.c_char_p, _D, _I, _D, _D, _D, _D, _D, _D, C.c_double, _I, _D, _D, C.c_int,
                               _D, _D, _D, _D]
    L.orc_initflow.restype = C.c_int
    L.orc_state_new.argtypes = [C.c_void_p]
    L.orc_state_new.restype = C.c_void_p
    L.orc_state_free.argtypes = [C.c_void_p]
    L.orc_state_ptr.argtypes = [C.c_void_p, C.c_int]
    L.orc_state_ptr.restype = _D
    L.orc_state_start.argtypes = [C.c_void_p]
    L.orc_state_step.argtypes = [C.c_void_p]
    L.orc_state_scalar.argtypes = [C.c_void_p, C.c_int]
    L.orc_state_scalar.restype = C.c_double
    L.orc_num_threads.restype = C.c_int
    L.orc_set_num_threads.argtypes = [C.c_int]


def _p(a):
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim <= 1), "need float64 Fortran array"
    return a.ctypes.data_as(_D)


def _ip(v):
    a = (C.c_int * len(v))(*[int(x) for x in v])
    return a


def _dp(v):
    return (C.c_double * len(v))(*[float(x) for x in v])


def _cs(chars):
    s = "".join(chars) if not isinstance(chars, (bytes, str)) else chars
    return s.encode() if isinstance(s, str) else s


def field(n):
    return np.zeros((n[0] + 2, n[1] + 2, n[2] + 2), dtype=np.float64, order="F")


def num_threads():
    return lib().orc_num_threads()


def set_num_threads(n):
    lib().orc_set_num_threads(int(n))


def initgrid(gtype, n, gr, lz, is_periodic):
    arrs = [np.zeros(n + 2) for _ in range(4)]
    rc = lib().orc_initgrid(gtype, n, gr, lz, int(is_periodic), *[_p(a) for a in arrs])
    if rc != 0:
        raise ValueError("unsupported grid type")
    dzc, dzf, zc, zf = arrs
    return dzc, dzf, zc, zf


def eigenvalues(n, bc, c_or_f):
    lam = np.zeros(n)
    lib().orc_eigenvalues(n, _cs(bc), _cs(c_or_f), _p(lam))
    return lam


def tridmatrix(bc, n, dzci, dzfi, c_or_f):
    a, b, c = np.zeros(n), np.zeros(n), np.zeros(n)
    lib().orc_tridmatrix(_cs(bc), n, _p(dzci), _p(dzfi), _cs(c_or_f), _p(a), _p(b), _p(c))
    return a, b, c


def initsolver(ng, dli, dzci_g, dzfi_g, cbc, bc, c_or_f):
    """cbc/bc: 6 entries in (ibound, idir) Fortran order."""
    lam = np.zeros((ng[0], ng[1]), order="F")
    a, b, c = np.zeros(ng[2]), np.zeros(ng[2]), np.zeros(ng[2])
    normfft = C.c_double(0.)
    rhsb = (C.c_double * 6)()
    lib().orc_initsolver(_ip(ng), _dp(dli), _p(dzci_g), _p(dzfi_g), _cs(cbc), _dp(bc), _cs(c_or_f),
                         _p(lam), _p(a), _p(b), _p(c), C.byref(normfft), rhsb)
    return dict(lambdaxy=lam, a=a, b=b, c=c, normfft=normfft.value, rhsb=np.array(list(rhsb)))


def r2r(kind, x):
    """FFTW r2r (unnormalised) along axis 0 of a 1D/2D float64 array (copy returned)."""
    y = np.array(x, dtype=np.float64, order="F", copy=True)
    n = y.shape[0]
    howmany = y.size // n
    rc = lib().orc_r2r(kind, n, howmany, 1, n, _p(y))
    if rc != 0:
        raise ValueError("bad r2r size")
    return y


def r2r_dir(kind, direction, nt, arr):
    nx, ny, nz = arr.shape
    lib().orc_r2r_dir(kind, direction, nt, nx, ny, nz, _p(arr))


def gaussel(a, b, c, is_periodic, norm, p, lambdaxy=None, n=None):
    nx, ny, nz = p.shape
    n = nz if n is None else n
    lib().orc_gaussel(nx, ny, n, nz, _p(a), _p(b), _p(c), int(is_periodic), norm, _p(p),
                      None if lambdaxy is None else _p(lambdaxy))


def solver(n, normfft, lambdaxy, a, b, c, cbc, c_or_f, p):
    lib().orc_solver(_ip(n), normfft, _p(lambdaxy), _p(a), _p(b), _p(c), _cs(cbc), _cs(c_or_f), _p(p))


def solve_helmholtz(n, normfft, alpha, lambdaxy, a, b, c, rhsb, is_bound, cbc, c_or_f, p):
    lib().orc_solve_helmholtz(_ip(n), normfft, alpha, _p(lambdaxy), _p(a), _p(b), _p(c), _dp(rhsb),
                              _ip(is_bound), _cs(cbc), _cs(c_or_f), _p(p))


def rk_buoy(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, dt, visc, p, is_forced, velf, bforce, is_impdiff, gacc, beta,
            s, dudtrko, dvdtrko, dwdtrko, u, v, w):
    """orc_rk_buoy: rk with the Boussinesq buoyancy of scalar s"""
    f = np.zeros(3)
    work = np.zeros(6 * n[0] * n[1] * n[2])
    lib().orc_rk_buoy(_dp(rkpar), _ip(n), _dp(dli), _p(dzci), _p(dzfi), _p(gvr_c), _p(gvr_f), float(dt), float(visc),
                      _p(p), _ip(is_forced), _dp(velf), _dp(bforce), int(is_impdiff), _dp(gacc), float(beta), _p(s),
                      _p(dudtrko), _p(dvdtrko), _p(dwdtrko), _p(u), _p(v), _p(w), _p(f), _p(work))
    return f


def rk_scal(rkpar, n, dli, dzci, dzfi, gvr_f, alpha, dt, u, v, w, is_forced, scalf, ssource, is_impdiff, dsdtrko, s):
    """orc_rk_scal: returns f"""
    work = np.zeros(2 * n[0] * n[1] * n[2])
    return lib().orc_rk_scal(_dp(rkpar), _ip(n), _dp(dli), _p(dzci), _p(dzfi), _p(gvr_f), float(alpha), float(dt),
                             _p(u), _p(v), _p(w), int(is_forced), float(scalf), float(ssource), int(is_impdiff),
                             _p(dsdtrko), _p(s), _p(work))


def bulk_forcing_s(n, is_forced, f, s):
    lib().orc_bulk_forcing_s(_ip(n), int(is_forced), float(f), _p(s))


def out1d(n, l, dl, idir, dz, p):
    out = np.zeros(n[idir - 1])
    lib().orc_out1d(_ip(n), _dp(l), _dp(dl), int(idir), _p(dz), _p(p), _p(out))
    return out


def out1d_chan(n, l, dl, u, v, w):
    out = np.zeros(7 * n[2])
    lib().orc_out1d_chan(_ip(n), _dp(l), _dp(dl), _p(u), _p(v), _p(w), _p(out))
    return out.reshape(7, n[2])


def out2d_duct(n, l, dl, idir, u, v, w):
    q = n[1] if idir == 1 else n[0]
    out = np.zeros(8 * q * n[2])
    lib().orc_out2d_duct(_ip(n), _dp(l), _dp(dl), int(idir), _p(u), _p(v), _p(w), _p(out))
    return out.reshape(8, n[2], q)


def fillps(n, dli, dzfi, dti, u, v, w, p):
    lib().orc_fillps(_ip(n), _dp(dli), _p(dzfi), dti, _p(u), _p(v), _p(w), _p(p))


def correc(n, dli, dzci, dt, p, u, v, w):
    lib().orc_correc(_ip(n), _dp(dli), _p(dzci), dt, _p(p), _p(u), _p(v), _p(w))


def updatep(n, dli, dzci, dzfi, alpha, is_impdiff, pp, p):
    lib().orc_updatep(_ip(n), _dp(dli), _p(dzci), _p(dzfi), alpha, int(is_impdiff), _p(pp), _p(p))


def mom_xyz_ad(n, dxi, dyi, dzci, dzfi, visc, u, v, w, is_impdiff=False):
    outs = [np.zeros(tuple(n), order="F") for _ in range(6)]
    lib().orc_mom_xyz_ad(_ip(n), dxi, dyi, _p(dzci), _p(dzfi), visc, _p(u), _p(v), _p(w),
                         *[_p(o) for o in outs], int(is_impdiff))
    return outs[:3] if not is_impdiff else outs


def bulk_mean(n, gvr, p):
    return lib().orc_bulk_mean(_ip(n), _p(gvr), _p(p))


def rk(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, dt, visc, p, is_forced, velf, bforce, is_impdiff,
       dudtrko, dvdtrko, dwdtrko, u, v, w):
    f = (C.c_double * 3)()
    work = np.zeros(6 * int(np.prod(n)))
    lib().orc_rk(_dp(rkpar), _ip(n), _dp(dli), _p(dzci), _p(dzfi), _p(gvr_c), _p(gvr_f), dt, visc, _p(p),
                 _ip(is_forced), _dp(velf), _dp(bforce), int(is_impdiff), _p(dudtrko), _p(dvdtrko),
                 _p(dwdtrko), _p(u), _p(v), _p(w), f, _p(work))
    return np.array(list(f))


def bounduvw(cbc, n, bc, is_bound, dl, dzc, dzf, u, v, w, keep_norm=False, halos_norm=HALO_BOTH,
             halos_tang=HALO_BOTH):
    lib().orc_bounduvw(_cs(cbc), _ip(n), _dp(bc), _ip(is_bound), _dp(dl), _p(dzc), _p(dzf), _p(u), _p(v),
                       _p(w), int(keep_norm), halos_norm, halos_tang)


def boundp(cbc, n, bc, is_bound, dl, dzc, p, halo_side=HALO_BOTH):
    lib().orc_boundp(_cs(cbc), _ip(n), _dp(bc), _ip(is_bound), _dp(dl), _p(dzc), _p(p), halo_side)


def updt_rhs_b(c_or_f, cbc, n, is_bound, rhsb, p, alpha=None):
    lib().orc_updt_rhs_b(_cs(c_or_f), _cs(cbc), _ip(n), _ip(is_bound), _dp(rhsb), _p(p),
                         0. if alpha is None else alpha, 0 if alpha is None else 1)


def chkdt(n, dl, dzci, dzfi, visc, alpha, is_impdiff, is_impdiff_1d, u, v, w):
    return lib().orc_chkdt(_ip(n), _dp(dl), _p(dzci), _p(dzfi), visc, alpha, int(is_impdiff),
                           int(is_impdiff_1d), _p(u), _p(v), _p(w))


def chkdiv(n, l, dli, dzfi, u, v, w):
    a, b = C.c_double(), C.c_double()
    lib().orc_chkdiv(_ip(n), _dp(l), _dp(dli), _p(dzfi), _p(u), _p(v), _p(w), C.byref(a), C.byref(b))
    return a.value, b.value


def poisson_residual_ld(n, dli, cbc, a, b, c, x, rhs):
    """rhs - L x in extended precision for the cell-centred Poisson operator (halo-free
    (n1, n2, n3) Fortran-ordered result); x, rhs haloed"""
    r = np.zeros(tuple(n), order="F")
    a, b, c = (np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, c))
    lib().orc_poisson_residual_ld(_ip(n), _dp(dli), _cs(cbc), _p(a), _p(b), _p(c), _p(x), _p(rhs), _p(r))
    return r


def initflow(inivel, bcvel, n, l, dl, zc, zf, dzc, dzf, visc, is_forced, velf, bforce, is_wallturb, u, v, w, p):
    """initflow (src/initflow.f90:16-259) into the interiors of the Fortran-ordered u, v, w, p"""
    rc = lib().orc_initflow(_cs(inivel), _dp(bcvel), _ip(n), _dp(l), _dp(dl), _p(np.ascontiguousarray(zc)),
                            _p(np.ascontiguousarray(zf)), _p(np.ascontiguousarray(dzc)),
                            _p(np.ascontiguousarray(dzf)), float(visc), _ip(is_forced), _dp(velf), _dp(bforce),
                            int(bool(is_wallturb)), _p(u), _p(v), _p(w), _p(p))
    if rc != 0:
        raise ValueError(f"initflow: unknown initial condition {inivel!r}")


def add_noise(n, seed, norm, p):
    lib().orc_add_noise(_ip(n), seed, norm, _p(p))


# ------------------------------------------------------------------------------------------------
class _Case(C.Structure):
    _fields_ = [("ng", C.c_int * 3), ("l", C.c_double * 3), ("gtype", C.c_int), ("gr", C.c_double),
                ("cfl", C.c_double), ("dtmax", C.c_double), ("dt_f", C.c_double), ("visci", C.c_double),
                ("icheck", C.c_int), ("cbcvel", C.c_char * 18), ("bcvel", C.c_double * 18),
                ("cbcpre", C.c_char * 6), ("bcpre", C.c_double * 6), ("bforce", C.c_double * 3),
                ("is_forced", C.c_int * 3), ("velf", C.c_double * 3), ("is_impdiff", C.c_int),
                ("nscal", C.c_int), ("alphai", C.c_double), ("cbcscal", C.c_char * 6), ("bcscal", C.c_double * 6),
                ("ssource", C.c_double), ("is_sforced", C.c_int), ("scalf", C.c_double), ("gacc", C.c_double * 3),
                ("beta", C.c_double), ("is_buoyancy", C.c_int)]


class Run:
    """Whole-run driver, one rank: src/main.f90 set-up and time loop without I/O.

    `case` is a dict with the input.nml keys used here (ng, l, gtype, gr, cfl, dtmax, dt_f,
    visci, icheck, cbcvel (18 chars), bcvel (18), cbcpre (6 chars), bcpre (6), bforce,
    is_forced, velf, is_impdiff) and, for one transported scalar, the &scalar keys nscal (0 or 1),
    alphai, cbcscal, bcscal, ssource, is_sforced, scalf, gacc, beta, is_boussinesq_buoyancy, each
    scalar entry given as a one-element list."""

    def __init__(self, case):
        cs = _Case()
        cs.ng[:] = case["ng"]
        cs.l[:] = case["l"]
        cs.gtype, cs.gr = case.get("gtype", 1), case.get("gr", 0.)
        cs.cfl, cs.dtmax, cs.dt_f = case.get("cfl", 0.95), case.get("dtmax", 1e5), case.get("dt_f", -1.)
        cs.visci, cs.icheck = case["visci"], case.get("icheck", 10)
        cs.cbcvel = _cs(case["cbcvel"])
        cs.bcvel[:] = case.get("bcvel", [0.] * 18)
        cs.cbcpre = _cs(case["cbcpre"])
        cs.bcpre[:] = case.get("bcpre", [0.] * 6)
        cs.bforce[:] = case.get("bforce", [0.] * 3)
        cs.is_forced[:] = [int(x) for x in case.get("is_forced", [0] * 3)]
        cs.velf[:] = case.get("velf", [0.] * 3)
        cs.is_impdiff = int(case.get("is_impdiff", 0))
        cs.nscal = min(1, max(0, int(case.get("nscal", 0))))
        if int(case.get("nscal", 0)) > 1:
            raise ValueError("the oracle run carries at most one scalar")
        if cs.nscal:
            cs.alphai = float(case["alphai"][0])
            cs.cbcscal = _cs(case["cbcscal"][0])
            cs.bcscal[:] = list(case.get("bcscal", [[0.] * 6])[0])
            cs.ssource = float(case.get("ssource", [0.])[0])
            cs.is_sforced = int(case.get("is_sforced", [0])[0])
            cs.scalf = float(case.get("scalf", [0.])[0])
        cs.gacc[:] = case.get("gacc", [0.] * 3)
        cs.beta = float(case.get("beta", 0.))
        cs.is_buoyancy = int(bool(case.get("is_boussinesq_buoyancy", False)))
        self._cs = cs
        self.n = list(case["ng"])
        self._h = lib().orc_state_new(C.byref(cs))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_state_free(self._h)
            self._h = None

    def array(self, which):
        n1, n2, n3 = self.n
        ptr = lib().orc_state_ptr(self._h, which)
        if which < 10:
            shape, count = (n1 + 2, n2 + 2, n3 + 2), (n1 + 2) * (n2 + 2) * (n3 + 2)
        elif which < 20:
            shape, count = (n3 + 2,), n3 + 2
        elif which == 20:
            shape, count = (n1, n2), n1 * n2
        else:
            shape, count = (n3,), n3
        buf = np.ctypeslib.as_array(ptr, shape=(count,))
        return buf.reshape(shape, order="F")

    u = property(lambda s: s.array(0))
    v = property(lambda s: s.array(1))
    w = property(lambda s: s.array(2))
    p = property(lambda s: s.array(3))
    pp = property(lambda s: s.array(4))
    s = property(lambda s: s.array(5))

    def grid(self):
        return {k: self.array(i) for k, i in
                (("dzc", 10), ("dzf", 11), ("zc", 12), ("zf", 13), ("dzci", 14), ("dzfi", 15))}

    def start(self):
        lib().orc_state_start(self._h)

    def step(self, nsteps=1):
        for _ in range(nsteps):
            lib().orc_state_step(self._h)

    def scalar(self, which):
        return lib().orc_state_scalar(self._h, which)

    time = property(lambda s: s.scalar(0))
    dt = property(lambda s: s.scalar(1))
    istep = property(lambda s: int(s.scalar(2)))
    divmax = property(lambda s: s.scalar(4))
    fs = property(lambda s: s.scalar(9))
