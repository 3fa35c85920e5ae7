"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this module.  It wraps

* ``libsctl_oracle.so`` -- the plain-C restatement of SCTL's GenericKernel
  Eval / KernelMatrix (sctl_oracle.c), and
* ``_ref/libsctlref.so`` -- the reference's own header-only implementation,
  wrapped by ref_driver.cpp (only present where the reference checkout was
  available at build time), and
* ``_ref/libsctlref_hot.so`` -- the reference's own Eval of the four hot-path
  kernels (ref_hot.cpp), built by ``make -C oracle hot`` wherever the
  reference is installed in baseline/_ref (also on the GPU host, where it is
  the timed CPU baseline).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libsctl_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsctlref.so")
REF_HOT_SO = os.path.join(HERE, "_ref", "libsctlref_hot.so")

KERNELS = {"Laplace3D_FxU": 0, "Laplace3D_DxU": 1, "Stokes3D_FxU": 2, "Stokes3D_DxU": 3,
           "Laplace3D_FxdU": 4, "Laplace3D_Fxd2U": 5, "Laplace3D_DxdU": 6, "BiotSavart3D_FxU": 7,
           "BiotSavart3D_FxdU": 8, "Helmholtz3D_FxU": 9, "Helmholtz3D_DxU": 10, "Helmholtz3D_FxdU": 11,
           "HelmholtzDiff3D_FxdU": 12, "Stokes3D_FxT": 13, "Stokes3D_FSxU": 14, "Stokes3D_FxUP": 15}
# (NormalDim, SrcDim, TrgDim), generic-kernel.hpp:54-74 with kernel_functions.hpp
DIMS = {0: (0, 1, 1), 1: (3, 1, 1), 2: (0, 3, 3), 3: (3, 3, 3), 4: (0, 1, 3), 5: (0, 1, 9), 6: (3, 1, 3),
        7: (0, 3, 3), 8: (0, 3, 9), 9: (0, 2, 2), 10: (3, 2, 2), 11: (0, 2, 6), 12: (0, 2, 6), 13: (0, 3, 9),
        14: (0, 4, 3), 15: (0, 3, 4)}
HELMHOLTZ = (9, 10, 11, 12)

_lib = None
_ref = None
_ref_hot = None


def build(force: bool = False) -> None:
    """Compile the oracle with gcc (seconds); never touches the product library."""
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(
            os.path.join(HERE, "sctl_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE, "libsctl_oracle.so"], check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(ORACLE_SO)
        i64, vp, i32 = ctypes.c_int64, ctypes.c_void_p, ctypes.c_int
        for name in ("oracle_eval_f64", "oracle_eval_f32", "oracle_eval_ld"):
            getattr(L, name).argtypes = [i32, i64, vp, i64, vp, vp, vp, vp, i32]
            getattr(L, name).restype = i32
        for name in ("oracle_kernel_matrix_f64", "oracle_kernel_matrix_f32"):
            getattr(L, name).argtypes = [i32, i64, vp, i64, vp, vp, vp, i32]
            getattr(L, name).restype = i32
        L.oracle_newton_steps.argtypes = [i32, i32, ctypes.c_double]
        L.oracle_newton_steps.restype = i32
        L.oracle_rsqrt_newton.argtypes = [ctypes.c_double, ctypes.c_double, i32]
        L.oracle_rsqrt_newton.restype = ctypes.c_double
        L.oracle_scale_factor.argtypes = [i32]
        L.oracle_scale_factor.restype = ctypes.c_double
        L.oracle_max_threads.restype = i32
        L.oracle_xscale.argtypes = [i32]
        L.oracle_xscale.restype = ctypes.c_double
        L.oracle_xeval.argtypes = [i32, i32, i64, vp, i64, vp, vp, vp, ctypes.c_double, vp, i32]
        L.oracle_xeval.restype = i32
        L.oracle_xkmat.argtypes = [i32, i32, i64, vp, i64, vp, vp, ctypes.c_double, vp, i32]
        L.oracle_xkmat.restype = i32
        L.oracle_near_pairs.argtypes = [i64, vp, i64, vp, vp, vp, vp, i64, vp, vp]
        L.oracle_near_pairs.restype = i64
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference wrapper not built (oracle/_ref/libsctlref.so)")
        L = ctypes.CDLL(REF_SO)
        i64, vp, i32 = ctypes.c_int64, ctypes.c_void_p, ctypes.c_int
        L.ref_eval.argtypes = [i32, i32, i32, i64, vp, i64, vp, vp, vp, vp, i32]
        L.ref_eval.restype = i32
        L.ref_kernel_matrix.argtypes = [i32, i32, i64, vp, i64, vp, vp, vp]
        L.ref_kernel_matrix.restype = i32
        L.ref_vec_len.argtypes = [i32]
        L.ref_vec_len.restype = i32
        L.ref_set_ctx.argtypes = [ctypes.c_double]
        L.ref_set_ctx.restype = None
        L.ref_near_list.argtypes = [i64, vp, i64, vp, vp, i64, vp, vp]
        L.ref_near_list.restype = i64
        L.ref_near_list_get.argtypes = [vp, vp, vp, vp, vp, vp]
        L.ref_near_list_get.restype = i32
        _ref = L
    return _ref


def ref_hot_available() -> bool:
    return os.path.exists(REF_HOT_SO)


def ref_hot():
    global _ref_hot
    if _ref_hot is None:
        if not ref_hot_available():
            raise RuntimeError("reference hot-kernel wrapper not built (oracle/_ref/libsctlref_hot.so)")
        L = ctypes.CDLL(REF_HOT_SO)
        i64, vp, i32 = ctypes.c_int64, ctypes.c_void_p, ctypes.c_int
        L.ref_hot_eval.argtypes = [i32, i32, i32, i64, vp, i64, vp, vp, vp, vp]
        L.ref_hot_eval.restype = i32
        L.ref_hot_threads.argtypes = []
        L.ref_hot_threads.restype = i32
        _ref_hot = L
    return _ref_hot


def ref_hot_eval(kernel, r_trg, r_src, n_src, v_src, digits=-1, precision="f64", v_trg=None):
    """The reference's own GenericKernel::Eval<Real,true>(..., digits, self) for kernel ids 0-3
    (oracle/_ref/libsctlref_hot.so); adds into v_trg when given."""
    k = _kid(kernel)
    if k > 3:
        raise ValueError("ref_hot_eval covers the four hot-path kernels (ids 0-3)")
    nd, sd, td = DIMS[k]
    dt = np.float32 if precision == "f32" else np.float64
    r_trg = np.ascontiguousarray(r_trg, dt).reshape(-1)
    r_src = np.ascontiguousarray(r_src, dt).reshape(-1)
    v_src = np.ascontiguousarray(v_src, dt).reshape(-1)
    n_src = np.ascontiguousarray(n_src, dt).reshape(-1) if nd else None
    nt, ns = r_trg.size // 3, r_src.size // 3
    if v_trg is None:
        v_trg = np.zeros(nt * td, dt)
    rc = ref_hot().ref_hot_eval(k, int(dt == np.float64), int(digits), nt, _ptr(r_trg), ns, _ptr(r_src),
                                _ptr(n_src), _ptr(v_src), _ptr(v_trg))
    if rc:
        raise RuntimeError(f"reference eval failed: {rc}")
    return v_trg


def ref_hot_threads() -> int:
    return ref_hot().ref_hot_threads()


def _kid(kernel):
    return KERNELS[kernel] if isinstance(kernel, str) else int(kernel)


def _ptr(a):
    return None if a is None or a.size == 0 else a.ctypes.data


def eval(kernel, r_trg, r_src, n_src, v_src, v_trg=None, precision="f64", nthreads=0, mu=0.0):
    """v_trg (+)= scale * sum_s K f (the reference's Eval); returns v_trg.  mu: the Helmholtz
    wavenumber (kernel ids 9-12)."""
    k = _kid(kernel)
    if k >= 4:
        return _xeval(k, r_trg, r_src, n_src, v_src, v_trg, precision, nthreads, mu)
    nd, sd, td = DIMS[k]
    dt = np.float32 if precision == "f32" else np.float64
    r_trg = np.ascontiguousarray(r_trg, dt).reshape(-1)
    r_src = np.ascontiguousarray(r_src, dt).reshape(-1)
    v_src = np.ascontiguousarray(v_src, dt).reshape(-1)
    n_src = np.ascontiguousarray(n_src, dt).reshape(-1) if nd else None
    nt, ns = r_trg.size // 3, r_src.size // 3
    if v_trg is None:
        v_trg = np.zeros(nt * td, dt)
    fn = {"f64": lib().oracle_eval_f64, "f32": lib().oracle_eval_f32, "ld": lib().oracle_eval_ld}[precision]
    rc = fn(k, nt, _ptr(r_trg), ns, _ptr(r_src), _ptr(n_src), _ptr(v_src), _ptr(v_trg), nthreads)
    if rc:
        raise RuntimeError(f"oracle eval failed: {rc}")
    return v_trg


def _xeval(k, r_trg, r_src, n_src, v_src, v_trg, precision, nthreads, mu):
    nd, sd, td = DIMS[k]
    dt = np.float32 if precision == "f32" else np.float64
    r_trg = np.ascontiguousarray(r_trg, dt).reshape(-1)
    r_src = np.ascontiguousarray(r_src, dt).reshape(-1)
    v_src = np.ascontiguousarray(v_src, dt).reshape(-1)
    n_src = np.ascontiguousarray(n_src, dt).reshape(-1) if nd else None
    nt, ns = r_trg.size // 3, r_src.size // 3
    if v_trg is None:
        v_trg = np.zeros(nt * td, dt)
    prec = {"f64": 0, "f32": 1, "ld": 2}[precision]
    rc = lib().oracle_xeval(k, prec, nt, _ptr(r_trg), ns, _ptr(r_src), _ptr(n_src), _ptr(v_src), float(mu),
                            _ptr(v_trg), nthreads)
    if rc:
        raise RuntimeError(f"oracle eval failed: {rc}")
    return v_trg


def kernel_matrix(kernel, r_trg, r_src, n_src, precision="f64", nthreads=0, mu=0.0):
    k = _kid(kernel)
    if k >= 4:
        nd, sd, td = DIMS[k]
        dt = np.float32 if precision == "f32" else np.float64
        r_trg = np.ascontiguousarray(r_trg, dt).reshape(-1)
        r_src = np.ascontiguousarray(r_src, dt).reshape(-1)
        n_src = np.ascontiguousarray(n_src, dt).reshape(-1) if nd else None
        nt, ns = r_trg.size // 3, r_src.size // 3
        M = np.zeros((ns * sd, nt * td), dt)
        rc = lib().oracle_xkmat(k, int(precision == "f32"), nt, _ptr(r_trg), ns, _ptr(r_src), _ptr(n_src),
                                float(mu), _ptr(M), nthreads)
        if rc:
            raise RuntimeError(f"oracle kernel_matrix failed: {rc}")
        return M
    nd, sd, td = DIMS[k]
    dt = np.float32 if precision == "f32" else np.float64
    r_trg = np.ascontiguousarray(r_trg, dt).reshape(-1)
    r_src = np.ascontiguousarray(r_src, dt).reshape(-1)
    n_src = np.ascontiguousarray(n_src, dt).reshape(-1) if nd else None
    nt, ns = r_trg.size // 3, r_src.size // 3
    M = np.zeros((ns * sd, nt * td), dt)
    fn = lib().oracle_kernel_matrix_f32 if precision == "f32" else lib().oracle_kernel_matrix_f64
    rc = fn(k, nt, _ptr(r_trg), ns, _ptr(r_src), _ptr(n_src), _ptr(M), nthreads)
    if rc:
        raise RuntimeError(f"oracle kernel_matrix failed: {rc}")
    return M


def ref_eval(kernel, r_trg, r_src, n_src, v_src, digits=-1, precision="f64", omp=True, v_trg=None, mu=0.0):
    """The reference's own GenericKernel::Eval<Real,omp>(..., digits, self)."""
    k = _kid(kernel)
    nd, sd, td = DIMS[k]
    dt = np.float32 if precision == "f32" else np.float64
    r_trg = np.ascontiguousarray(r_trg, dt).reshape(-1)
    r_src = np.ascontiguousarray(r_src, dt).reshape(-1)
    v_src = np.ascontiguousarray(v_src, dt).reshape(-1)
    n_src = np.ascontiguousarray(n_src, dt).reshape(-1) if nd else None
    nt, ns = r_trg.size // 3, r_src.size // 3
    if v_trg is None:
        v_trg = np.zeros(nt * td, dt)
    ref().ref_set_ctx(float(mu))
    rc = ref().ref_eval(k, int(dt == np.float64), int(digits), nt, _ptr(r_trg), ns, _ptr(r_src), _ptr(n_src),
                        _ptr(v_src), _ptr(v_trg), int(omp))
    if rc:
        raise RuntimeError(f"reference eval failed: {rc}")
    return v_trg


def ref_kernel_matrix(kernel, r_trg, r_src, n_src, precision="f64", mu=0.0):
    k = _kid(kernel)
    nd, sd, td = DIMS[k]
    dt = np.float32 if precision == "f32" else np.float64
    r_trg = np.ascontiguousarray(r_trg, dt).reshape(-1)
    r_src = np.ascontiguousarray(r_src, dt).reshape(-1)
    n_src = np.ascontiguousarray(n_src, dt).reshape(-1) if nd else None
    nt, ns = r_trg.size // 3, r_src.size // 3
    M = np.zeros((ns * sd, nt * td), dt)
    ref().ref_set_ctx(float(mu))
    rc = ref().ref_kernel_matrix(k, int(dt == np.float64), nt, _ptr(r_trg), ns, _ptr(r_src), _ptr(n_src), _ptr(M))
    if rc:
        raise RuntimeError(f"reference kernel_matrix failed: {rc}")
    return M


def newton_steps(digits, is_double, seed_digits):
    return lib().oracle_newton_steps(int(digits), int(is_double), float(seed_digits))


def rsqrt_newton(x, y0, steps):
    return lib().oracle_rsqrt_newton(float(x), float(y0), int(steps))


def scale_factor(kernel):
    k = _kid(kernel)
    return lib().oracle_xscale(k) if k >= 4 else lib().oracle_scale_factor(k)


def max_threads():
    return lib().oracle_max_threads()


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def max_rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


# ------------------------------------------------------------------ near lists
def near_pairs(r_trg, elem_nds_cnt, elem_nds_dsp, r_src, src_radius):
    """Element-major (element, target) near pairs by brute force (sctl_oracle.c oracle_near_pairs)."""
    xt = np.ascontiguousarray(r_trg, np.float64).reshape(-1)
    xs = np.ascontiguousarray(r_src, np.float64).reshape(-1)
    rad = np.ascontiguousarray(src_radius, np.float64)
    cnt = np.ascontiguousarray(elem_nds_cnt, np.int64)
    dsp = np.ascontiguousarray(elem_nds_dsp, np.int64)
    L = lib()
    args = (xt.size // 3, _ptr(xt), cnt.size, _ptr(cnt), _ptr(dsp), _ptr(xs), _ptr(rad))
    n = L.oracle_near_pairs(*args, 0, None, None)
    pe, pt = np.empty(max(n, 1), np.int64), np.empty(max(n, 1), np.int64)
    m = L.oracle_near_pairs(*args, n, pe.ctypes.data, pt.ctypes.data)
    assert m == n
    return pe[:n], pt[:n]


def near_list_from_pairs(pe, pt, nt, n_elem):
    """BuildNearList's outputs (boundary_integral.txx:423-521) from element-major sorted pairs:
    near_elem_cnt/dsp, near_trg_idx, near_scatter_index (target-major order, ties in element
    order), near_trg_cnt/dsp (dsp 0 where cnt is 0)."""
    elem_cnt = np.bincount(pe, minlength=n_elem).astype(np.int64)
    elem_dsp = np.concatenate([[0], np.cumsum(elem_cnt)[:-1]]).astype(np.int64)
    scatter = np.argsort(pt, kind="stable").astype(np.int64)
    trg_cnt = np.bincount(pt, minlength=nt).astype(np.int64)
    trg_dsp = np.concatenate([[0], np.cumsum(trg_cnt)[:-1]]).astype(np.int64)
    trg_dsp[trg_cnt == 0] = 0
    return dict(near_elem_cnt=elem_cnt, near_elem_dsp=elem_dsp[:n_elem], near_trg_idx=pt.astype(np.int64),
                near_scatter_index=scatter, near_trg_cnt=trg_cnt, near_trg_dsp=trg_dsp)


def ref_near_list(r_trg, elem_nds_cnt, elem_nds_dsp, r_src, src_radius):
    """The reference's own BuildNearList<double,3> on one rank (oracle/_ref)."""
    xt = np.ascontiguousarray(r_trg, np.float64).reshape(-1)
    xs = np.ascontiguousarray(r_src, np.float64).reshape(-1)
    rad = np.ascontiguousarray(src_radius, np.float64)
    cnt = np.ascontiguousarray(elem_nds_cnt, np.int64)
    dsp = np.ascontiguousarray(elem_nds_dsp, np.int64)
    nt, ne = xt.size // 3, cnt.size
    L = ref()
    n = L.ref_near_list(nt, _ptr(xt), ne, _ptr(cnt), _ptr(dsp), xs.size // 3, _ptr(xs), _ptr(rad))
    out = dict(xtrg_near=np.zeros(max(n, 1) * 3), near_elem_cnt=np.zeros(max(ne, 1), np.int64),
               near_elem_dsp=np.zeros(max(ne, 1), np.int64), near_scatter_index=np.zeros(max(n, 1), np.int64),
               near_trg_cnt=np.zeros(max(nt, 1), np.int64), near_trg_dsp=np.zeros(max(nt, 1), np.int64))
    L.ref_near_list_get(*(out[k].ctypes.data for k in ("xtrg_near", "near_elem_cnt", "near_elem_dsp",
                                                       "near_scatter_index", "near_trg_cnt", "near_trg_dsp")))
    out["xtrg_near"] = out["xtrg_near"][:n * 3].reshape(-1, 3)
    out["near_elem_cnt"], out["near_elem_dsp"] = out["near_elem_cnt"][:ne], out["near_elem_dsp"][:ne]
    out["near_scatter_index"] = out["near_scatter_index"][:n]
    out["near_trg_cnt"], out["near_trg_dsp"] = out["near_trg_cnt"][:nt], out["near_trg_dsp"][:nt]
    return out
