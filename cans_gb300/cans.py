"""Python host mirror of the CaNS routines on the pressure-correction path.

Binds the C ABI of libcans_gb300.so (include/cans_gb300.h) with ctypes.  The
function names, argument order and meaning follow the reference Fortran
routines (src/initsolver.f90, src/solver_gpu.f90, src/fillps.f90, ...); device
memory comes from torch (plumbing only: every computation runs in the library's
own CUDA kernels).  There is no CPU fallback: importing this module on a
machine without the built library raises.

Field layout: haloed fields are torch float64 CUDA tensors of shape
(n3+2, n2+2, n1+2) -- the same bytes as the reference's Fortran arrays
p(0:n1+1, 0:n2+1, 0:n3+1).  `fview(t)` returns the Fortran-indexed numpy view
[i, j, k] of a tensor copied to the host.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

OK, EINVAL, ENOMEM, ECUDA, ENOTSUP, ETIMEOUT, ENONFINITE, EIO = range(8)
FP64, FP32 = 0, 1
HALO_LOWER, HALO_NONE, HALO_UPPER, HALO_BOTH = -1, 0, 1, 2

_lib = None
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_V = C.c_void_p


class CansError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        super().__init__(f"{where}: {lib().cans_strerror(status).decode()} (status {status})")


def lib_path():
    return _build.LIB


def lib():
    """Load libcans_gb300.so (building it first if this tree has nvcc and no library)."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            path = _build.build()
        _lib = C.CDLL(path)
        _setup(_lib)
    return _lib


class CBox(C.Structure):
    """struct cans_box of include/cans_gb300.h"""
    _fields_ = [("n", C.c_int * 3), ("l", C.c_double * 3), ("visc", C.c_double), ("dt", C.c_double),
                ("cbcvel", C.c_char * 18), ("cbcpre", C.c_char * 6), ("bcvel", C.c_double * 18),
                ("bcpre", C.c_double * 6), ("bforce", C.c_double * 3), ("dzc_g", _D), ("dzf_g", _D),
                ("dzci", _V), ("dzfi", _V), ("u", _V), ("v", _V), ("w", _V), ("p", _V), ("pp", _V),
                ("dudtrko", _V), ("dvdtrko", _V), ("dwdtrko", _V)]


def _setup(L):
    L.cans_strerror.restype = C.c_char_p
    L.cans_strerror.argtypes = [C.c_int]
    L.cans_version.restype = C.c_char_p
    L.cans_initgrid.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, _D, _D, _D, _D]
    L.cans_initsolver.argtypes = [_I, _D, _D, _D, C.c_char_p, _D, C.c_char_p, C.c_int, _V, C.POINTER(_V),
                                  _D, _D, _D, _D, _D, _D]
    L.cans_plan_destroy.argtypes = [_V]
    L.cans_plan_device_bytes.argtypes = [_V]
    L.cans_plan_device_bytes.restype = C.c_longlong
    L.cans_plan_set_timing.argtypes = [_V, C.c_int]
    L.cans_plan_get_timing.argtypes = [_V, _D, _I]
    L.cans_plan_get_residual_timing.argtypes = [_V, _D, _I]
    L.cans_launch_count.restype = C.c_longlong
    L.cans_solver.argtypes = [_V, _V]
    L.cans_solver_f32.argtypes = [_V, _V]
    L.cans_solver_refined.argtypes = [_V, _V, _D, _V, _V, C.c_double, C.c_int, _I, _D]
    L.cans_solve_helmholtz.argtypes = [_V, C.c_double, _I, _V]
    L.cans_fillps.argtypes = [_I, _D, _V, C.c_double, _V, _V, _V, _V, _V]
    L.cans_correc.argtypes = [_I, _D, _V, C.c_double, _V, _V, _V, _V, _V]
    L.cans_updatep.argtypes = [_I, _D, _V, _V, C.c_double, C.c_int, _V, _V, _V]
    L.cans_rk.argtypes = [_D, _I, _D, _V, _V, _V, _V, C.c_double, C.c_double, _V, _I, _D, _D, C.c_int,
                          _V, _V, _V, _V, _V, _V, _D, _V, _V]
    L.cans_bounduvw.argtypes = [C.c_char_p, _I, _D, _I, _D, _D, _D, _V, _V, _V, C.c_int, C.c_int, C.c_int, _V]
    L.cans_boundp.argtypes = [C.c_char_p, _I, _D, _I, _D, _D, _V, C.c_int, _V]
    L.cans_updt_rhs_b.argtypes = [C.c_char_p, C.c_char_p, _I, _I, _D, _V, C.c_double, C.c_int, _V]
    L.cans_chkdiv.argtypes = [_I, _D, _D, _V, _V, _V, _V, _D, _D, _V]
    L.cans_chkdt.argtypes = [_I, _D, _V, _V, C.c_double, C.c_double, C.c_int, C.c_int, _V, _V, _V, _D, _V]
    L.cans_bulk_mean.argtypes = [_I, _V, _V, _D, _V]
    L.cans_batch_create.argtypes = [C.c_int, C.POINTER(_V), _V, C.POINTER(_V)]
    L.cans_batch_destroy.argtypes = [_V]
    L.cans_batch_solve.argtypes = [_V, C.POINTER(_V), _D, _I]
    L.cans_boxes_create.argtypes = [C.c_int, C.POINTER(CBox), C.c_int, C.c_int, _V, C.POINTER(_V)]
    L.cans_plan_autotune.argtypes = [_V, C.c_int, _D]
    L.cans_rk_buoy.argtypes = [_D, _I, _D, _V, _V, _V, _V, C.c_double, C.c_double, _V, _I, _D, _D, C.c_int, _D,
                               C.c_double, _V, _V, _V, _V, _V, _V, _V, _D, _V, _V]
    L.cans_rk_scal.argtypes = [_D, _I, _D, _V, _V, _V, C.c_double, C.c_double, _V, _V, _V, C.c_int, C.c_double,
                               C.c_double, C.c_int, _V, _V, _D, _V, _V]
    L.cans_rk_scal_work_doubles.argtypes = [_I, C.c_int]
    L.cans_rk_scal_work_doubles.restype = C.c_size_t
    L.cans_bulk_forcing_s.argtypes = [_I, C.c_int, C.c_double, _V, _V]
    L.cans_save_field.argtypes = [C.c_char_p, _I, _V, C.c_double, C.c_int, _V]
    L.cans_out1d.argtypes = [_I, _D, _D, C.c_int, _V, _V, _V, _V]
    L.cans_out1d_chan.argtypes = [_I, _D, _D, C.c_int, _V, _V, _V, _V, _V]
    L.cans_out2d_duct.argtypes = [_I, _D, _D, C.c_int, _V, _V, _V, _V, _V]
    L.cans_load_field.argtypes = [C.c_char_p, _I, _V, _D, _I, _V]
    L.cans_solver_adjoint.argtypes = [_V, _V]
    L.cans_solve_helmholtz_adjoint.argtypes = [_V, C.c_double, _V]
    L.cans_fillps_adjoint.argtypes = [_I, _D, _V, C.c_double, _V, _V, _V, _V, _V]
    L.cans_correc_adjoint.argtypes = [_I, _D, _V, C.c_double, _V, _V, _V, _V, _V]
    L.cans_updatep_adjoint.argtypes = [_I, _D, _V, _V, C.c_double, C.c_int, _V, _V, _V]
    L.cans_bounduvw_adjoint.argtypes = [C.c_char_p, _I, _D, _I, _D, _D, _D, _V, _V, _V, C.c_int, C.c_int, C.c_int, _V]
    L.cans_boundp_adjoint.argtypes = [C.c_char_p, _I, _D, _I, _D, _D, _V, C.c_int, _V]
    L.cans_rk_adjoint.argtypes = [_D, _I, _D, _V, _V, C.c_double, C.c_double, C.c_int, _V, _V, _V, _V, _V, _V, _V,
                                  _V, _V, _V, _D, _V, _V]
    L.cans_rk_adjoint_work_doubles.argtypes = [_I]
    L.cans_rk_adjoint_work_doubles.restype = C.c_size_t
    L.cans_plan_get_shape.argtypes = [_V, C.c_int, _I, _I, _I, _I]
    L.cans_boxes_destroy.argtypes = [_V]
    L.cans_boxes_start.argtypes = [_V]
    L.cans_boxes_substep.argtypes = [_V, C.c_int]
    L.cans_boxes_step.argtypes = [_V, C.c_int]
    L.cans_boxes_graph_nodes.argtypes = [_V]
    L.cans_boxes_graph_nodes.restype = C.c_longlong
    # the FP32 run
    L.cans_fillps_f32.argtypes = [_I, _D, _V, C.c_double, _V, _V, _V, _V, _V]
    L.cans_correc_f32.argtypes = [_I, _D, _V, C.c_double, _V, _V, _V, _V, _V]
    L.cans_updatep_f32.argtypes = [_I, _D, _V, _V, C.c_double, C.c_int, _V, _V, _V]
    L.cans_rk_f32.argtypes = [_D, _I, _D, _V, _V, _V, _V, C.c_double, C.c_double, _V, _I, _D, _D, C.c_int,
                              _V, _V, _V, _V, _V, _V, _V, _V, _V, _D, _V, _V]
    L.cans_rk_f32_work_bytes.argtypes = [_I, C.c_int]
    L.cans_rk_f32_work_bytes.restype = C.c_size_t
    L.cans_bounduvw_f32.argtypes = L.cans_bounduvw.argtypes
    L.cans_boundp_f32.argtypes = L.cans_boundp.argtypes
    L.cans_chkdiv_f32.argtypes = L.cans_chkdiv.argtypes
    L.cans_chkdt_f32.argtypes = L.cans_chkdt.argtypes
    L.cans_bulk_mean_f32.argtypes = L.cans_bulk_mean.argtypes
    L.cans_correc_updatep_f32.argtypes = [_I, _D, _V, C.c_double, _V, _V, _V, _V, _V, _V]
    L.cans_selftest_wait_timeout.argtypes = [C.c_int, _I]
    L.cans_plan_set_zpass.argtypes = [_V, C.c_int]
    L.cans_plan_check.argtypes = [_V]
    L.cans_initflow.argtypes = [C.c_char_p, _D, _I, _D, _D, _D, _D, _D, _D, C.c_double, _I, _D, _D, C.c_int,
                                _V, _V, _V, _V, _V]
    L.cans_plan_get_zpass.argtypes = [_V, _I]


def _check(rc, where):
    if rc != OK:
        raise CansError(rc, where)


def _ints(v):
    return (C.c_int * len(v))(*[int(x) for x in v])


def _dbls(v):
    return (C.c_double * len(v))(*[float(x) for x in v])


def _chars(s):
    return s.encode() if isinstance(s, str) else bytes(s)


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _hp(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_D)


def _stream(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


# ------------------------------------------------------------------------------ fields
def field(n, device="cuda", dtype=None):
    import torch
    return torch.zeros((n[2] + 2, n[1] + 2, n[0] + 2), dtype=dtype or torch.float64, device=device)


def to_device(arr_f, device="cuda", dtype=None):
    """Fortran-indexed numpy array [i, j, k] -> device tensor (k, j, i)."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(arr_f).transpose(2, 1, 0))).to(
        device=device, dtype=dtype or torch.float64)


def fview(t):
    """device tensor (k, j, i) -> Fortran-indexed numpy array [i, j, k] (host copy)."""
    return t.detach().cpu().numpy().transpose(2, 1, 0)


# ------------------------------------------------------------------------------ solver plan
class Plan:
    """initsolver + the device plan (src/initsolver.f90:15, src/fft.f90:25)."""

    def __init__(self, ng, dli, dzci_g, dzfi_g, cbc, bc, c_or_f="ccc", precision=FP64, stream=None):
        ng = [int(x) for x in ng]
        self.ng = ng
        self.cbc, self.c_or_f = cbc, c_or_f
        self.lambdaxy = np.zeros((ng[0], ng[1]), order="F")
        self.a, self.b, self.c = np.zeros(ng[2]), np.zeros(ng[2]), np.zeros(ng[2])
        normfft = C.c_double()
        rhsb = (C.c_double * 6)()
        h = C.c_void_p()
        dzci_g, pzc = _hp(dzci_g)
        dzfi_g, pzf = _hp(dzfi_g)
        rc = lib().cans_initsolver(_ints(ng), _dbls(dli), pzc, pzf, _chars(cbc), _dbls(bc), _chars(c_or_f),
                                   int(precision), _stream(stream), C.byref(h),
                                   self.lambdaxy.ctypes.data_as(_D), self.a.ctypes.data_as(_D),
                                   self.b.ctypes.data_as(_D), self.c.ctypes.data_as(_D), C.byref(normfft), rhsb)
        _check(rc, "cans_initsolver")
        self._h = h
        self.normfft = normfft.value
        self.rhsb = np.array(list(rhsb))
        self.precision = precision

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.cans_plan_destroy(h)
            self._h = None

    @property
    def device_bytes(self):
        return lib().cans_plan_device_bytes(self._h)

    def set_timing(self, enable=True):
        _check(lib().cans_plan_set_timing(self._h, int(enable)), "cans_plan_set_timing")

    def get_timing(self):
        """mean ms per pass (x-fwd, y-fwd, z, y-bwd, x-bwd) over the solves since the last call"""
        ms = (C.c_double * 5)()
        cnt = C.c_int()
        _check(lib().cans_plan_get_timing(self._h, ms, C.byref(cnt)), "cans_plan_get_timing")
        return list(ms), cnt.value

    def get_residual_timing(self):
        """mean ms of the refinement's residual launches since timing was enabled, and their count"""
        ms, cnt = C.c_double(), C.c_int()
        _check(lib().cans_plan_get_residual_timing(self._h, C.byref(ms), C.byref(cnt)),
               "cans_plan_get_residual_timing")
        return ms.value, cnt.value

    def solve(self, p):
        """solver (src/solver_gpu.f90:34) in place on a haloed float64 (or float32) field."""
        import torch
        if p.dtype == torch.float32:
            _check(lib().cans_solver_f32(self._h, _ptr(p)), "cans_solver_f32")
        else:
            _check(lib().cans_solver(self._h, _ptr(p)), "cans_solver")
        return p

    def solve_refined(self, p, dli, dzci, dzfi, rtol=1e-13, max_iter=6):
        it, rr = C.c_int(), C.c_double()
        _check(lib().cans_solver_refined(self._h, _ptr(p), _dbls(dli), _ptr(dzci), _ptr(dzfi), rtol, max_iter,
                                         C.byref(it), C.byref(rr)), "cans_solver_refined")
        return it.value, rr.value

    def autotune(self, force=False):
        """cans_plan_autotune: fastest x/y transform shapes; returns the chosen pass times (ms)"""
        ms = (C.c_double * 2)()
        _check(lib().cans_plan_autotune(self._h, int(force), ms), "cans_plan_autotune")
        return list(ms)

    def check(self):
        """cans_plan_check: True when the solves since the last check were all finite"""
        rc = lib().cans_plan_check(self._h)
        if rc == ENONFINITE:
            return False
        _check(rc, "cans_plan_check")
        return True

    @property
    def zpass(self):
        """z pass of an FP32 plan: 0 column sweep, 1 partitioned, 2 TMA-tiled (cans_plan_get_zpass)"""
        m = C.c_int()
        _check(lib().cans_plan_get_zpass(self._h, C.byref(m)), "cans_plan_get_zpass")
        return m.value

    def set_zpass(self, mode):
        """cans_plan_set_zpass: 0 column sweep, 1 partitioned, 2 TMA-tiled, -1 automatic"""
        _check(lib().cans_plan_set_zpass(self._h, int(mode)), "cans_plan_set_zpass")

    def shape(self, d):
        """(radix order, lines per CTA, compile-time length or 0) of direction d"""
        r = (C.c_int * 12)()
        ns, ncx, spec = C.c_int(), C.c_int(), C.c_int()
        _check(lib().cans_plan_get_shape(self._h, int(d), r, C.byref(ns), C.byref(ncx), C.byref(spec)),
               "cans_plan_get_shape")
        return list(r)[:ns.value], ncx.value, spec.value

    def solve_adjoint(self, g):
        """S^T g in place (cans_solver_adjoint)"""
        _check(lib().cans_solver_adjoint(self._h, _ptr(g)), "cans_solver_adjoint")
        return g

    def solve_helmholtz_adjoint(self, alpha, g):
        _check(lib().cans_solve_helmholtz_adjoint(self._h, float(alpha), _ptr(g)), "cans_solve_helmholtz_adjoint")
        return g

    def solve_helmholtz(self, alpha, is_bound, p):
        """solve_helmholtz (src/solve_helmholtz.f90:28), 3D variant."""
        _check(lib().cans_solve_helmholtz(self._h, float(alpha), _ints(is_bound), _ptr(p)), "cans_solve_helmholtz")
        return p


class Batch:
    """Independent solves of many plans in one persistent launch per pass (cans_batch_*).

    `solve(fields, alpha=None, is_bound=None)`: system s is the Helmholtz solve of
    `plans[s].solve_helmholtz(alpha[s], is_bound[s], fields[s])` when alpha[s] != 0, else
    `updt_rhs_b` (when is_bound is given) followed by `plans[s].solve(fields[s])`."""

    def __init__(self, plans, stream=None):
        self.plans = list(plans)
        hs = (_V * len(self.plans))(*[pl._h.value for pl in self.plans])
        h = C.c_void_p()
        _check(lib().cans_batch_create(len(self.plans), hs, _stream(stream), C.byref(h)), "cans_batch_create")
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib is not None:
            _lib.cans_batch_destroy(h)
            self._h = None

    def solve(self, fields, alpha=None, is_bound=None):
        ns = len(self.plans)
        if len(fields) != ns:
            raise ValueError("one field per system")
        ps = (_V * ns)(*[f.data_ptr() for f in fields])
        al = None if alpha is None else _dbls(alpha)
        ib = None if is_bound is None else _ints([int(x) for b in is_bound for x in b])
        _check(lib().cans_batch_solve(self._h, ps, al, ib), "cans_batch_solve")
        return fields


# ------------------------------------------------------------------------------ kernels
def launch_count():
    return lib().cans_launch_count()


def fillps(n, dli, dzfi, dti, u, v, w, p, stream=None):
    _check(lib().cans_fillps(_ints(n), _dbls(dli), _ptr(dzfi), float(dti), _ptr(u), _ptr(v), _ptr(w), _ptr(p),
                             _stream(stream)), "cans_fillps")


def correc(n, dli, dzci, dt, p, u, v, w, stream=None):
    _check(lib().cans_correc(_ints(n), _dbls(dli), _ptr(dzci), float(dt), _ptr(p), _ptr(u), _ptr(v), _ptr(w),
                             _stream(stream)), "cans_correc")


def updatep(n, dli, dzci, dzfi, alpha, is_impdiff, pp, p, stream=None):
    _check(lib().cans_updatep(_ints(n), _dbls(dli), _ptr(dzci), _ptr(dzfi), float(alpha), int(is_impdiff), _ptr(pp),
                              _ptr(p), _stream(stream)), "cans_updatep")


def rk(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, dt, visc, p, is_forced, velf, bforce, is_impdiff,
       dudtrko, dvdtrko, dwdtrko, u, v, w, work=None, stream=None):
    f = (C.c_double * 3)()
    _check(lib().cans_rk(_dbls(rkpar), _ints(n), _dbls(dli), _ptr(dzci), _ptr(dzfi), _ptr(gvr_c), _ptr(gvr_f),
                         float(dt), float(visc), _ptr(p), _ints(is_forced), _dbls(velf), _dbls(bforce),
                         int(is_impdiff), _ptr(dudtrko), _ptr(dvdtrko), _ptr(dwdtrko), _ptr(u), _ptr(v), _ptr(w),
                         f, _ptr(work), _stream(stream)), "cans_rk")
    return np.array(list(f))


def bounduvw(cbc, n, bc, is_bound, dl, dzc_h, dzf_h, u, v, w, keep_norm=False, halos_norm=HALO_BOTH,
             halos_tang=HALO_BOTH, stream=None):
    dzc_h, pc = _hp(dzc_h)
    dzf_h, pf = _hp(dzf_h)
    _check(lib().cans_bounduvw(_chars(cbc), _ints(n), _dbls(bc), _ints(is_bound), _dbls(dl), pc, pf, _ptr(u),
                               _ptr(v), _ptr(w), int(keep_norm), int(halos_norm), int(halos_tang), _stream(stream)),
           "cans_bounduvw")


def boundp(cbc, n, bc, is_bound, dl, dzc_h, p, halo_side=HALO_BOTH, stream=None):
    dzc_h, pc = _hp(dzc_h)
    _check(lib().cans_boundp(_chars(cbc), _ints(n), _dbls(bc), _ints(is_bound), _dbls(dl), pc, _ptr(p),
                             int(halo_side), _stream(stream)), "cans_boundp")


def updt_rhs_b(c_or_f, cbc, n, is_bound, rhsb, p, alpha=None, stream=None):
    _check(lib().cans_updt_rhs_b(_chars(c_or_f), _chars(cbc), _ints(n), _ints(is_bound), _dbls(rhsb), _ptr(p),
                                 0. if alpha is None else float(alpha), 0 if alpha is None else 1, _stream(stream)),
           "cans_updt_rhs_b")


def chkdiv(n, l, dli, dzfi, u, v, w, stream=None, allow_nonfinite=False):
    """chkdiv (src/chkdiv.f90:15): (divtot, divmax).  A non-finite result raises CansError
    (CANS_ENONFINITE) unless allow_nonfinite, which returns the values as they are."""
    a, b = C.c_double(), C.c_double()
    rc = lib().cans_chkdiv(_ints(n), _dbls(l), _dbls(dli), _ptr(dzfi), _ptr(u), _ptr(v), _ptr(w), C.byref(a),
                           C.byref(b), _stream(stream))
    if not (allow_nonfinite and rc == ENONFINITE):
        _check(rc, "cans_chkdiv")
    return a.value, b.value


def chkdt(n, dl, dzci, dzfi, visc, alpha, is_impdiff, is_impdiff_1d, u, v, w, stream=None):
    r = C.c_double()
    _check(lib().cans_chkdt(_ints(n), _dbls(dl), _ptr(dzci), _ptr(dzfi), float(visc), float(alpha), int(is_impdiff),
                            int(is_impdiff_1d), _ptr(u), _ptr(v), _ptr(w), C.byref(r), _stream(stream)), "cans_chkdt")
    return r.value


def bulk_mean(n, gvr, p, stream=None):
    r = C.c_double()
    _check(lib().cans_bulk_mean(_ints(n), _ptr(gvr), _ptr(p), C.byref(r), _stream(stream)), "cans_bulk_mean")
    return r.value


# ------------------------------------------------------------------------------ adjoints
def fillps_adjoint(n, dli, dzfi, dti, gp, gu, gv, gw, stream=None):
    _check(lib().cans_fillps_adjoint(_ints(n), _dbls(dli), _ptr(dzfi), float(dti), _ptr(gp), _ptr(gu), _ptr(gv),
                                     _ptr(gw), _stream(stream)), "cans_fillps_adjoint")


def correc_adjoint(n, dli, dzci, dt, gu, gv, gw, gp, stream=None):
    _check(lib().cans_correc_adjoint(_ints(n), _dbls(dli), _ptr(dzci), float(dt), _ptr(gu), _ptr(gv), _ptr(gw),
                                     _ptr(gp), _stream(stream)), "cans_correc_adjoint")


def updatep_adjoint(n, is_impdiff, gp, gpp, dli=None, dzci=None, dzfi=None, alpha=0., stream=None):
    """updatep^T: gpp += gp (explicit) or gpp += (I + alpha lap)^T gp (is_impdiff; needs dli,
    dzci, dzfi and alpha as given to updatep)"""
    _check(lib().cans_updatep_adjoint(_ints(n), _dbls(dli) if dli is not None else None,
                                      _ptr(dzci) if dzci is not None else None,
                                      _ptr(dzfi) if dzfi is not None else None, float(alpha), int(is_impdiff),
                                      _ptr(gp), _ptr(gpp), _stream(stream)), "cans_updatep_adjoint")


def bounduvw_adjoint(cbc, n, bc, is_bound, dl, dzc_h, dzf_h, gu, gv, gw, keep_norm=False, halos_norm=HALO_BOTH,
                     halos_tang=HALO_BOTH, stream=None):
    dzc_h, pzc = _hp(dzc_h)
    dzf_h, pzf = _hp(dzf_h)
    _check(lib().cans_bounduvw_adjoint(_chars(cbc), _ints(n), _dbls(bc), _ints(is_bound), _dbls(dl), pzc, pzf,
                                       _ptr(gu), _ptr(gv), _ptr(gw), int(keep_norm), int(halos_norm),
                                       int(halos_tang), _stream(stream)), "cans_bounduvw_adjoint")


def boundp_adjoint(cbc, n, bc, is_bound, dl, dzc_h, gp, halo_side=HALO_BOTH, stream=None):
    dzc_h, pzc = _hp(dzc_h)
    _check(lib().cans_boundp_adjoint(_chars(cbc), _ints(n), _dbls(bc), _ints(is_bound), _dbls(dl), pzc, _ptr(gp),
                                     int(halo_side), _stream(stream)), "cans_boundp_adjoint")


def rk_adjoint_work(n, device="cuda"):
    import torch
    return torch.empty(int(lib().cans_rk_adjoint_work_doubles(_ints(n))), dtype=torch.float64, device=device)


def rk_adjoint(rkpar, n, dli, dzci, dzfi, dt, visc, u, v, w, gu, gv, gw, gdu, gdv, gdw, gp, work, want_gbf=True,
               stream=None, is_impdiff=0):
    """returns the body-force adjoint increment (3,) when want_gbf"""
    gbf = (C.c_double * 3)()
    _check(lib().cans_rk_adjoint(_dbls(rkpar), _ints(n), _dbls(dli), _ptr(dzci), _ptr(dzfi), float(dt), float(visc),
                                 int(is_impdiff), _ptr(u), _ptr(v), _ptr(w), _ptr(gu), _ptr(gv), _ptr(gw), _ptr(gdu), _ptr(gdv),
                                 _ptr(gdw), _ptr(gp), gbf if want_gbf else None, _ptr(work), _stream(stream)),
           "cans_rk_adjoint")
    return np.array(list(gbf))


# ------------------------------------------------------------------------------ profile statistics
def _stats_out(count, like):
    import torch
    return torch.empty(int(count), dtype=torch.float64, device=like.device)


def out1d(n, l, dl, idir, dz, p, stream=None):
    """out1d (src/output.f90:56-157): the profile of p along idir averaged over the other
    two directions (device tensor of n[idir-1] values).  dz: device dzf/dzc (0..n3+1)."""
    out = _stats_out(n[idir - 1], p)
    _check(lib().cans_out1d(_ints(n), _dbls(l), _dbls(dl), int(idir), _ptr(dz), _ptr(p), _ptr(out),
                            _stream(stream)), "cans_out1d")
    return out


def out1d_chan(n, l, dl, u, v, w, idir=3, stream=None):
    """out1d_chan (src/output.f90:327-393): (7, n3) device tensor um, vm, wm, u2, v2, w2, uw."""
    out = _stats_out(7 * n[2], u)
    _check(lib().cans_out1d_chan(_ints(n), _dbls(l), _dbls(dl), int(idir), _ptr(u), _ptr(v), _ptr(w), _ptr(out),
                                 _stream(stream)), "cans_out1d_chan")
    return out.view(7, n[2])


def out2d_duct(n, l, dl, idir, u, v, w, stream=None):
    """out2d_duct (src/output.f90:395-529): (8, n3, q) device tensor, q = n2 (idir 1) or n1
    (idir 2); rows um, vm, wm, u2, v2, w2 and uv, uw (idir 1) or vw, uv (idir 2)."""
    q = n[1] if idir == 1 else n[0]
    out = _stats_out(8 * q * n[2], u)
    _check(lib().cans_out2d_duct(_ints(n), _dbls(l), _dbls(dl), int(idir), _ptr(u), _ptr(v), _ptr(w), _ptr(out),
                                 _stream(stream)), "cans_out2d_duct")
    return out.view(8, n[2], q)


# ------------------------------------------------------------------------------ checkpoints
def save_field(path, n, p, time, istep, stream=None):
    """load_one('w', ...) (src/load.f90:461): interior in Fortran order + [time, istep]."""
    _check(lib().cans_save_field(str(path).encode(), _ints(n), _ptr(p), float(time), int(istep), _stream(stream)),
           "cans_save_field")


def load_field(path, n, p, stream=None):
    """load_one('r', ...): fills the interior of p, returns (time, istep)."""
    t, it = C.c_double(), C.c_int()
    _check(lib().cans_load_field(str(path).encode(), _ints(n), _ptr(p), C.byref(t), C.byref(it), _stream(stream)),
           "cans_load_field")
    return t.value, it.value


def read_field_file(path, n):
    """Host reader of a checkpoint file (the layout of the reference's
    utils/read_binary_data/python/read_single_field_binary.py): returns the Fortran-indexed
    interior array [i, j, k], time and istep."""
    a = np.fromfile(path, dtype=np.float64)
    npts = n[0] * n[1] * n[2]
    if a.size != npts + 2:
        raise ValueError(f"{path}: {a.size} values, expected {npts + 2}")
    return a[:npts].reshape((n[0], n[1], n[2]), order="F"), float(a[npts]), int(round(a[npts + 1]))


# ------------------------------------------------------------------------------ scalars
def rk_buoy(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, dt, visc, p, is_forced, velf, bforce, is_impdiff, gacc, beta,
            s, dudtrko, dvdtrko, dwdtrko, u, v, w, work=None, stream=None):
    f = (C.c_double * 3)()
    _check(lib().cans_rk_buoy(_dbls(rkpar), _ints(n), _dbls(dli), _ptr(dzci), _ptr(dzfi), _ptr(gvr_c), _ptr(gvr_f),
                              float(dt), float(visc), _ptr(p), _ints(is_forced), _dbls(velf), _dbls(bforce),
                              int(is_impdiff), _dbls(gacc), float(beta), _ptr(s), _ptr(dudtrko), _ptr(dvdtrko),
                              _ptr(dwdtrko), _ptr(u), _ptr(v), _ptr(w), f, _ptr(work), _stream(stream)),
           "cans_rk_buoy")
    return np.array(list(f))


def rk_scal_work(n, is_impdiff, device="cuda"):
    import torch
    return torch.empty(int(lib().cans_rk_scal_work_doubles(_ints(n), int(is_impdiff))), dtype=torch.float64,
                       device=device)


def rk_scal(rkpar, n, dli, dzci, dzfi, gvr_f, alpha, dt, u, v, w, is_forced, scalf, ssource, is_impdiff, dsdtrko, s,
            work, stream=None):
    """rk_scal (src/rk.f90:335): returns f (scalf - mean when forced)"""
    f = C.c_double()
    _check(lib().cans_rk_scal(_dbls(rkpar), _ints(n), _dbls(dli), _ptr(dzci), _ptr(dzfi), _ptr(gvr_f), float(alpha),
                              float(dt), _ptr(u), _ptr(v), _ptr(w), int(is_forced), float(scalf), float(ssource),
                              int(is_impdiff), _ptr(dsdtrko), _ptr(s), C.byref(f), _ptr(work), _stream(stream)),
           "cans_rk_scal")
    return f.value


def bulk_forcing_s(n, is_forced, f, s, stream=None):
    _check(lib().cans_bulk_forcing_s(_ints(n), int(is_forced), float(f), _ptr(s), _stream(stream)),
           "cans_bulk_forcing_s")


# ------------------------------------------------------------------------------ the FP32 run
# The same routines on float32 fields and float32 device grid arrays; pp stays float64 (the
# refined solve's right-hand side and solution).
def fillps_f32(n, dli, dzfi, dti, u, v, w, p, stream=None):
    _check(lib().cans_fillps_f32(_ints(n), _dbls(dli), _ptr(dzfi), float(dti), _ptr(u), _ptr(v), _ptr(w), _ptr(p),
                                 _stream(stream)), "cans_fillps_f32")


def correc_f32(n, dli, dzci, dt, p, u, v, w, stream=None):
    _check(lib().cans_correc_f32(_ints(n), _dbls(dli), _ptr(dzci), float(dt), _ptr(p), _ptr(u), _ptr(v), _ptr(w),
                                 _stream(stream)), "cans_correc_f32")


def updatep_f32(n, dli, dzci, dzfi, alpha, is_impdiff, pp, p, stream=None):
    _check(lib().cans_updatep_f32(_ints(n), _dbls(dli), _ptr(dzci), _ptr(dzfi), float(alpha), int(is_impdiff),
                                  _ptr(pp), _ptr(p), _stream(stream)), "cans_updatep_f32")


def rk_f32_work(n, in_place=False, device="cuda"):
    import torch
    nb = int(lib().cans_rk_f32_work_bytes(_ints(n), int(bool(in_place))))
    return torch.empty(nb, dtype=torch.uint8, device=device)


def rk_f32(rkpar, n, dli, dzci, dzfi, gvr_c, gvr_f, dt, visc, p, is_forced, velf, bforce, dudtrko, dvdtrko,
           dwdtrko, u, v, w, unew, vnew, wnew, work, stream=None):
    """rk + mom_xyz_ad on FP32 fields; out of place into (unew, vnew, wnew) unless they are u, v, w"""
    f = (C.c_double * 3)()
    _check(lib().cans_rk_f32(_dbls(rkpar), _ints(n), _dbls(dli), _ptr(dzci), _ptr(dzfi), _ptr(gvr_c), _ptr(gvr_f),
                             float(dt), float(visc), _ptr(p), _ints(is_forced), _dbls(velf), _dbls(bforce), 0,
                             _ptr(dudtrko), _ptr(dvdtrko), _ptr(dwdtrko), _ptr(u), _ptr(v), _ptr(w), _ptr(unew),
                             _ptr(vnew), _ptr(wnew), f, _ptr(work), _stream(stream)), "cans_rk_f32")
    return np.array(list(f))


def bounduvw_f32(cbc, n, bc, is_bound, dl, dzc_h, dzf_h, u, v, w, keep_norm=False, halos_norm=HALO_BOTH,
                 halos_tang=HALO_BOTH, stream=None):
    dzc_h, pc = _hp(dzc_h)
    dzf_h, pf = _hp(dzf_h)
    _check(lib().cans_bounduvw_f32(_chars(cbc), _ints(n), _dbls(bc), _ints(is_bound), _dbls(dl), pc, pf, _ptr(u),
                                   _ptr(v), _ptr(w), int(keep_norm), int(halos_norm), int(halos_tang),
                                   _stream(stream)), "cans_bounduvw_f32")


def boundp_f32(cbc, n, bc, is_bound, dl, dzc_h, p, halo_side=HALO_BOTH, stream=None):
    dzc_h, pc = _hp(dzc_h)
    _check(lib().cans_boundp_f32(_chars(cbc), _ints(n), _dbls(bc), _ints(is_bound), _dbls(dl), pc, _ptr(p),
                                 int(halo_side), _stream(stream)), "cans_boundp_f32")


def chkdiv_f32(n, l, dli, dzfi, u, v, w, stream=None, allow_nonfinite=False):
    a, b = C.c_double(), C.c_double()
    rc = lib().cans_chkdiv_f32(_ints(n), _dbls(l), _dbls(dli), _ptr(dzfi), _ptr(u), _ptr(v), _ptr(w), C.byref(a),
                               C.byref(b), _stream(stream))
    if not (allow_nonfinite and rc == ENONFINITE):
        _check(rc, "cans_chkdiv_f32")
    return a.value, b.value


def chkdt_f32(n, dl, dzci, dzfi, visc, alpha, is_impdiff, is_impdiff_1d, u, v, w, stream=None):
    r = C.c_double()
    _check(lib().cans_chkdt_f32(_ints(n), _dbls(dl), _ptr(dzci), _ptr(dzfi), float(visc), float(alpha),
                                int(is_impdiff), int(is_impdiff_1d), _ptr(u), _ptr(v), _ptr(w), C.byref(r),
                                _stream(stream)), "cans_chkdt_f32")
    return r.value


def bulk_mean_f32(n, gvr, p, stream=None):
    r = C.c_double()
    _check(lib().cans_bulk_mean_f32(_ints(n), _ptr(gvr), _ptr(p), C.byref(r), _stream(stream)), "cans_bulk_mean_f32")
    return r.value


def correc_updatep_f32(n, dli, dzci, dt, pp, u, v, w, p, stream=None):
    """correc + the explicit updatep in one pass over pp (cans_correc_updatep_f32)"""
    _check(lib().cans_correc_updatep_f32(_ints(n), _dbls(dli), _ptr(dzci), float(dt), _ptr(pp), _ptr(u), _ptr(v),
                                         _ptr(w), _ptr(p), _stream(stream)), "cans_correc_updatep_f32")


def initflow(inivel, bcvel, n, l, dl, zc, zf, dzc, dzf, visc, is_forced, velf, bforce, is_wallturb, u, v, w, p,
             stream=None):
    """initflow (src/initflow.f90:16): interiors of the FP64 device fields u, v, w, p"""
    zc, pzc = _hp(zc)
    zf, pzf = _hp(zf)
    dzc, pdc = _hp(dzc)
    dzf, pdf = _hp(dzf)
    _check(lib().cans_initflow(_chars(inivel), _dbls(bcvel), _ints(n), _dbls(l), _dbls(dl), pzc, pzf, pdc, pdf,
                               float(visc), _ints(is_forced), _dbls(velf), _dbls(bforce), int(bool(is_wallturb)),
                               _ptr(u), _ptr(v), _ptr(w), _ptr(p), _stream(stream)), "cans_initflow")


def selftest_wait_timeout(limit_us=20000):
    """cans_selftest_wait_timeout: True when a bounded device wait that nothing releases gave up
    after limit_us and the kernel returned (the context stays usable)"""
    r = C.c_int(0)
    _check(lib().cans_selftest_wait_timeout(int(limit_us), C.byref(r)), "cans_selftest_wait_timeout")
    return bool(r.value)
