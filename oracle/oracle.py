"""ctypes front end of the C oracle and of the reference harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product path.

* `Oracle` wraps oracle/cfd_oracle.c (the FP64 restatement, built into
  oracle/_build/libcfd_oracle.so by `build_oracle()`).
* `RefHarness` wraps oracle/_ref/<workload>/libref.so, the reference's own
  headers driven by oracle/ref_harness.cpp (built by oracle/build_ref.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libcfd_oracle.so"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "cfd_oracle.c"
    BUILD.mkdir(exist_ok=True)
    if LIB.exists() and not force and LIB.stat().st_mtime > max(
            src.stat().st_mtime, (HERE / "cfd_oracle.h").stat().st_mtime):
        return LIB
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                    "-o", str(tmp), str(src), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


def p(a):
    """Pointer to the data of a contiguous numpy array (None -> NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be contiguous"
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_ip)
    raise TypeError(a.dtype)


class OgGrid(C.Structure):
    _fields_ = [("nxc", C.c_int), ("nyc", C.c_int), ("nzc", C.c_int),
                ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("X", _dp), ("Y", _dp), ("Z", _dp),
                ("Dx", _dp), ("Dy", _dp), ("Dz", _dp),
                ("Dxs", _dp), ("Dys", _dp), ("Dzs", _dp), ("periodic_z", C.c_int)]


class OgStepCfg(C.Structure):
    _fields_ = [("method", C.c_int), ("solver", C.c_int), ("aligned_src", C.c_int),
                ("compat", C.c_int), ("dt", C.c_double), ("nu", C.c_double),
                ("tol", C.c_double), ("omega", C.c_double), ("maxit", C.c_int),
                ("sor_maxit", C.c_int), ("conv_uc", C.c_double)]


class Grid:
    """Uniform staggered grid metrics (numpy) plus the C view of them."""

    def __init__(self, nxc, nyc, nzc, lx, ly, lz, oracle=None, metrics=None, periodic_z=False):
        self.nxc, self.nyc, self.nzc = nxc, nyc, nzc
        self.nx, self.ny, self.nz = nxc + 4, nyc + 4, nzc + 4
        self.lx, self.ly, self.lz = lx, ly, lz
        self.ng = self.nx * self.ny * self.nz
        self.n = nxc * nyc * nzc
        if metrics is None:
            metrics = {k: np.zeros(n) for k, n in
                       (("X", self.nx + 1), ("Y", self.ny + 1), ("Z", self.nz + 1),
                        ("Dx", self.nx), ("Dy", self.ny), ("Dz", self.nz),
                        ("Dxs", self.nx), ("Dys", self.ny), ("Dzs", self.nz))}
            (oracle or Oracle()).lib.og_grid_uniform(
                nxc, nyc, nzc, C.c_double(lx), C.c_double(ly), C.c_double(lz),
                *[p(metrics[k]) for k in ("X", "Y", "Z", "Dx", "Dy", "Dz", "Dxs", "Dys", "Dzs")])
        self.m = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in metrics.items()}
        self.periodic_z = bool(periodic_z)
        self.c = OgGrid(nxc, nyc, nzc, self.nx, self.ny, self.nz, lx, ly, lz,
                        *[p(self.m[k]) for k in ("X", "Y", "Z", "Dx", "Dy", "Dz", "Dxs", "Dys", "Dzs")],
                        int(self.periodic_z))

    @classmethod
    def of(cls, w, oracle=None, periodic_z=False):
        return cls(w.nxc, w.nyc, w.nzc, w.lx, w.ly, w.lz, oracle=oracle, periodic_z=periodic_z)

    def ref(self):
        return C.byref(self.c)

    def zeros(self):
        return np.zeros(self.ng)

    def interior(self, a):
        """View of the interior block of a ghosted array as (nxc, nyc, nzc)."""
        return a.reshape(self.nx, self.ny, self.nz)[2:-2, 2:-2, 2:-2]


class Oracle:
    def __init__(self):
        build_oracle()
        self.lib = L = C.CDLL(str(LIB))
        d, i, v = C.c_double, C.c_int, None
        L.og_dot.restype = d
        L.og_div_inf.restype = d
        L.og_rhs_compat.restype = d
        L.og_bicg_create.restype = C.c_void_p
        L.og_bicg_create.argtypes = [C.c_longlong, d, i]
        L.og_bicg_destroy.argtypes = [C.c_void_p]
        L.og_bicg_set_spe.argtypes = [C.c_void_p, i, i, i] + [_dp] * 7
        L.og_bicg_set_ell.argtypes = [C.c_void_p, _ip, _dp]
        L.og_bicg_solve.argtypes = [C.c_void_p, _dp, _dp, _ip, _dp]
        L.og_bicg_counters.argtypes = [C.c_void_p, _ip, _ip, _ip, _ip]
        L.og_sim_create.restype = C.c_void_p
        L.og_sim_create.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp, _dp]
        L.og_sim_destroy.argtypes = [C.c_void_p]
        L.og_sim_field.restype = _dp
        L.og_sim_field.argtypes = [C.c_void_p, i]
        L.og_sim_init.argtypes = [C.c_void_p, d, d, d]
        L.og_sim_start.argtypes = [C.c_void_p]
        L.og_sim_step.argtypes = [C.c_void_p, _ip, _dp, _dp, _dp]
        L.og_sim_loop.restype = C.c_longlong
        L.og_sim_loop.argtypes = [C.c_void_p]
        L.og_sim_set_loop.argtypes = [C.c_void_p, C.c_longlong]
        L.og_bc_convective.argtypes = [C.c_void_p, d, d] + [_dp] * 6
        del v

    # -- single kernels -------------------------------------------------
    def convdiff(self, g, dt, nu, u0, v0, w0, u1, v1, w1):
        self.lib.og_convdiff(g.ref(), C.c_double(dt), C.c_double(nu), p(u0), p(v0), p(w0),
                             p(u1), p(v1), p(w1))

    def convdiff_les(self, g, dt, nu, vis, u0, v0, w0, u1, v1, w1):
        self.lib.og_convdiff_les(g.ref(), C.c_double(dt), C.c_double(nu), p(vis), p(u0), p(v0), p(w0),
                                 p(u1), p(v1), p(w1))

    def smagorinsky(self, g, u, v, w):
        vis = np.zeros(g.n)
        self.lib.og_smagorinsky(g.ref(), p(u), p(v), p(w), p(vis))
        return vis

    def src_add(self, g, aligned, u1, v1, w1, src):
        self.lib.og_src_add(g.ref(), int(aligned), p(u1), p(v1), p(w1), p(src))

    def src_accumulate(self, g, dt, src, f):
        self.lib.og_src_accumulate(g.ref(), C.c_double(dt), p(src), p(f))

    def rhs(self, g, dt, jp, u1, v1, w1, b, compat=False):
        fn = self.lib.og_rhs_compat if compat else self.lib.og_rhs
        return fn(g.ref(), C.c_double(dt), p(jp), p(u1), p(v1), p(w1), p(b))

    def spe_setup(self, g):
        co = {k: np.zeros(n) for k, n in (("xm", g.nxc), ("xp", g.nxc), ("ym", g.nyc),
                                           ("yp", g.nyc), ("zm", g.nzc), ("zp", g.nzc))}
        val, jp = np.zeros(g.n), np.zeros(g.n)
        self.lib.og_spe_setup(g.ref(), *[p(co[k]) for k in ("xm", "xp", "ym", "yp", "zm", "zp")],
                              p(val), p(jp))
        return co, val, jp

    def spe_spmv(self, g, co, jp, x, r):
        self.lib.og_spe_spmv(g.nxc, g.nyc, g.nzc,
                             *[p(co[k]) for k in ("xm", "xp", "ym", "yp", "zm", "zp")],
                             p(jp), p(x), p(r))

    def ell_assemble(self, g):
        cols = np.zeros(7 * g.n, dtype=np.int32)
        vals = np.zeros(7 * g.n)
        jp = np.zeros(g.n)
        self.lib.og_ell_assemble(g.ref(), p(cols), p(vals), p(jp))
        return cols, vals, jp

    def ell_spmv(self, n, cols, vals, x, r):
        self.lib.og_ell_spmv(C.c_longlong(n), p(cols), p(vals), p(x), p(r))

    def sor_coef(self, g):
        cf = np.zeros(8 * g.n)
        self.lib.og_sor_coef(g.ref(), p(cf))
        return cf

    def sor_rhs(self, g, dt, u1, v1, w1, cf):
        self.lib.og_sor_rhs(g.ref(), C.c_double(dt), p(u1), p(v1), p(w1), p(cf))

    def sor(self, g, omega, tol, itmax, cf, pr, redblack=False):
        it, err = C.c_int(), C.c_double()
        fn = self.lib.og_sor_redblack if redblack else self.lib.og_sor_seq
        fn(g.ref(), C.c_double(omega), C.c_double(tol), int(itmax), p(cf), p(pr), C.byref(it),
           C.byref(err))
        return it.value, err.value

    def pressure_transform(self, g, x, pr):
        self.lib.og_pressure_transform(g.ref(), p(x), p(pr))

    def update_uf(self, g, dt, pr, eta, u1, v1, w1, u3, v3, w3, f):
        self.lib.og_update_uf(g.ref(), C.c_double(dt), p(pr), p(eta), p(u1), p(v1), p(w1),
                              p(u3), p(v3), p(w3), p(f))

    def cdcl(self, g, f):
        cd, cl = C.c_double(), C.c_double()
        self.lib.og_cdcl(g.ref(), p(f), C.byref(cd), C.byref(cl))
        return cd.value, cl.value

    def bc_main(self, g, bc_dir, bc_num, u, v, w, pr):
        d = np.ascontiguousarray(bc_dir, dtype=np.float64).ravel()
        n = np.ascontiguousarray(bc_num, dtype=np.float64).ravel()
        self.lib.og_bc_main(g.ref(), p(d), p(n), p(u), p(v), p(w), p(pr))

    def bc_convective(self, g, dt, uc, u0, v0, w0, u3, v3, w3):
        """Convective outflow at the x-max face (extension; og_bc_convective)."""
        self.lib.og_bc_convective(g.ref(), dt, uc, p(u0), p(v0), p(w0), p(u3), p(v3), p(w3))

    def bc_copy(self, g, uo, vo, wo, u, v, w):
        self.lib.og_bc_copy(g.ref(), p(uo), p(vo), p(wo), p(u), p(v), p(w))

    def eta_cylinder_z(self, g, cx, cy, radius=0.5, nsub=100):
        eta = np.zeros(g.ng)
        self.lib.og_eta_cylinder_z(g.ref(), C.c_double(cx), C.c_double(cy), C.c_double(radius),
                                   int(nsub), p(eta))
        return eta

    def div_inf(self, g, u, v, w):
        return self.lib.og_div_inf(g.ref(), p(u), p(v), p(w))

    def dot(self, a, b):
        return self.lib.og_dot(p(a), p(b), C.c_longlong(a.size))

    # -- monitors ---------------------------------------------------------
    def cfl(self, g, dt, u, v, w, umax=None, umin=None, cfl_max=-1e300):
        """(cfl, umax, umin, cfl_max); umax/umin/cfl_max are running values."""
        umax = np.full(3, -1e10) if umax is None else np.array(umax, dtype=np.float64)
        umin = np.full(3, 1e10) if umin is None else np.array(umin, dtype=np.float64)
        cm = C.c_double(cfl_max)
        L = self.lib
        L.og_cfl.restype = C.c_double
        L.og_cfl.argtypes = [C.c_void_p, C.c_double] + [_dp] * 5 + [_dp]
        c = L.og_cfl(g.ref(), dt, p(u), p(v), p(w), p(umax), p(umin), C.byref(cm))
        return c, umax, umin, cm.value

    def timestepper(self, re, umax, umin, cfl_factor=0.05, grid_fo_factor=0.15, dt_min=1e-12):
        L = self.lib
        L.og_timestepper.restype = C.c_double
        L.og_timestepper.argtypes = [C.c_double, _dp, _dp, C.c_double, C.c_double, C.c_double]
        return L.og_timestepper(re, p(np.asarray(umax, dtype=np.float64)), p(np.asarray(umin, dtype=np.float64)),
                                cfl_factor, grid_fo_factor, dt_min)

    def steady_max(self, g, u0, v0, w0, u3, v3, w3):
        out = np.zeros(3)
        self.lib.og_steady_max(g.ref(), p(u0), p(v0), p(w0), p(u3), p(v3), p(w3), p(out))
        return out

    # -- BiCGSTAB ---------------------------------------------------------
    class Bicg:
        def __init__(self, orc, g, tol, maxit=5000, spe=None, ell=None):
            self.L = orc.lib
            self.h = self.L.og_bicg_create(g.n, tol, maxit)
            self._keep = (spe, ell)
            if ell is not None:
                cols, vals = ell
                self.L.og_bicg_set_ell(self.h, p(cols), p(vals))
            else:
                co, jp = spe
                self.L.og_bicg_set_spe(self.h, g.nxc, g.nyc, g.nzc,
                                       *[p(co[k]) for k in ("xm", "xp", "ym", "yp", "zm", "zp")],
                                       p(jp))

        def solve(self, b, x):
            it, res = C.c_int(), C.c_double()
            capped = self.L.og_bicg_solve(self.h, p(b), p(x), C.byref(it), C.byref(res))
            return it.value, res.value, capped

        def counters(self):
            a = [C.c_int() for _ in range(4)]
            self.L.og_bicg_counters(self.h, *[C.byref(x) for x in a])
            return [x.value for x in a]

        def __del__(self):
            try:
                self.L.og_bicg_destroy(self.h)
            except Exception:
                pass

    def bicg(self, g, tol, maxit=5000, spe=None, ell=None):
        return Oracle.Bicg(self, g, tol, maxit, spe=spe, ell=ell)

    # -- whole step -------------------------------------------------------
    class Sim:
        FIELDS = {"u0": 0, "v0": 1, "w0": 2, "u1": 3, "v1": 4, "w1": 5, "u3": 6, "v3": 7,
                  "w3": 8, "p": 9, "eta": 10, "f": 11, "src": 12, "x": 13, "b": 14, "jp": 15}

        def __init__(self, orc, g, *, method=0, solver=0, aligned_src=False, compat=False,
                     dt, nu, tol, omega=1.7, maxit=5000, sor_maxit=5000, bc_dir, bc_num, eta,
                     conv_uc=0.0):
            self.L = orc.lib
            self.g = g
            cfg = OgStepCfg(method, solver, int(aligned_src), int(compat), dt, nu, tol, omega,
                            maxit, sor_maxit, conv_uc)
            d = np.ascontiguousarray(bc_dir, dtype=np.float64).ravel()
            n = np.ascontiguousarray(bc_num, dtype=np.float64).ravel()
            self.h = self.L.og_sim_create(C.addressof(g.c), C.addressof(cfg), p(d), p(n), p(eta))
            if not self.h:
                raise ValueError("og_sim_create refused the configuration (periodic z needs a Krylov solver)")

        def field(self, name):
            k = self.FIELDS[name]
            g = self.g
            n = g.ng if k <= 10 else (3 * g.n if k <= 12 else g.n)
            ptr = self.L.og_sim_field(self.h, k)
            return np.ctypeslib.as_array(ptr, shape=(n,))

        def init(self, ui=1.0, vi=0.0, wi=0.0):
            self.L.og_sim_init(self.h, ui, vi, wi)

        def start(self):
            self.L.og_sim_start(self.h)

        def step(self):
            it = (C.c_int * 4)()
            er = (C.c_double * 4)()
            cd, cl = C.c_double(), C.c_double()
            self.L.og_sim_step(self.h, it, er, C.byref(cd), C.byref(cl))
            return cd.value, cl.value, list(it), list(er)

        @property
        def loop(self):
            return self.L.og_sim_loop(self.h)

        @loop.setter
        def loop(self, v):
            self.L.og_sim_set_loop(self.h, C.c_longlong(int(v)))

        def __del__(self):
            try:
                self.L.og_sim_destroy(self.h)
            except Exception:
                pass

    def sim(self, g, **kw):
        return Oracle.Sim(self, g, **kw)


class RefHarness:
    """The reference's own functions (oracle/_ref/<name>/libref.so)."""

    def __init__(self, name: str, build: bool = True, fast: bool = False):
        """fast: the timing build (the reference's -O3 -march=native), when
        it exists; self.flags names the flags of the library loaded."""
        lib = HERE / "_ref" / name / "libref.so"
        self.flags = "-O2 -ffp-contract=off"
        if build:
            from oracle.build_ref import build as _build  # noqa: WPS433
            lib = _build(name)
        if fast:
            fl = HERE / "_ref" / name / "libref_fast.so"
            if fl.exists():
                lib = fl
                ff = HERE / "_ref" / name / "libref_fast.flags"
                self.flags = ff.read_text().strip() if ff.exists() else "-O3"
        if not lib.exists():
            raise FileNotFoundError(lib)
        self.L = L = C.CDLL(str(lib))
        d = C.c_double
        L.ref_setup.argtypes = [d, d, d, C.c_int]
        L.ref_cdcl.argtypes = [_dp, _dp, _dp]
        L.ref_sor_seq.argtypes = [_dp, _dp, _dp, _dp, d, d, C.c_int, _ip, _dp]
        L.ref_pc_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _dp]
        nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
        lens = (C.c_double * 3)()
        L.ref_dims(C.byref(nx), C.byref(ny), C.byref(nz), lens)
        self.nxc, self.nyc, self.nzc = nx.value, ny.value, nz.value
        self.lens = tuple(lens)
        self.ng = (self.nxc + 4) * (self.nyc + 4) * (self.nzc + 4)
        self.n = self.nxc * self.nyc * self.nzc

    def set_threads(self, n: int):
        self.L.ref_set_threads(int(n))

    def plot3d_x(self, directory):
        """OutputPlot3D_Xfile into directory/mx_out/P3D.x (the directory must exist)."""
        (Path(directory) / "mx_out").mkdir(exist_ok=True)
        assert self.L.ref_plot3d_x(str(directory).encode()) == 0
        return Path(directory) / "mx_out" / "P3D.x"

    def plot3d_q(self, directory, io, time, pr, u, v, w, eta):
        """OutputPLOT3D_Qfile of the given ghosted fields into
        directory/mx_out/P3D<io>.q."""
        (Path(directory) / "mx_out").mkdir(exist_ok=True)
        L = self.L
        L.ref_plot3d_q.argtypes = [C.c_char_p, C.c_int, C.c_double] + [_dp] * 5
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (pr, u, v, w, eta)]
        assert L.ref_plot3d_q(str(directory).encode(), int(io), float(time), *[p(a) for a in arrs]) == 0
        return Path(directory) / "mx_out" / f"P3D{io:02d}.q"

    def cfl(self, u, v, w):
        """get_Cfl of one field: (cfl, U_max[3], U_min[3]) of this call."""
        L = self.L
        L.ref_cfl.argtypes = [_dp] * 6
        c = np.zeros(1)
        umax, umin = np.zeros(3), np.zeros(3)
        L.ref_cfl(p(u), p(v), p(w), p(c), p(umax), p(umin))
        return c[0], umax, umin

    def timestepper(self, umax, umin):
        L = self.L
        L.ref_timestepper.restype = C.c_double
        L.ref_timestepper.argtypes = [_dp, _dp]
        return L.ref_timestepper(p(np.asarray(umax, dtype=np.float64)), p(np.asarray(umin, dtype=np.float64)))

    def steady_max(self, u0, v0, w0, u3, v3, w3):
        L = self.L
        L.ref_steady.argtypes = [_dp] * 7
        out = np.zeros(3)
        L.ref_steady(p(u0), p(v0), p(w0), p(u3), p(v3), p(w3), p(out))
        return out

    def plot3d_read(self, path):
        """QfileRead: ((mach, alpha, Re, time), p, u, v, w, eta) ghosted."""
        L = self.L
        L.ref_plot3d_read.argtypes = [C.c_char_p] + [_dp] * 6
        cond = np.zeros(4)
        out = [np.zeros(self.ng) for _ in range(5)]
        L.ref_plot3d_read(str(path).encode(), p(cond), *[p(a) for a in out])
        return (tuple(cond), *out)

    def setup(self, dt, re, tol=1e-3, with_eta=True):
        self.L.ref_setup(dt, re, tol, int(with_eta))

    def grid_metrics(self):
        nx, ny, nz = self.nxc + 4, self.nyc + 4, self.nzc + 4
        m = {k: np.zeros(n) for k, n in (("X", nx + 1), ("Y", ny + 1), ("Z", nz + 1),
                                          ("Dx", nx), ("Dy", ny), ("Dz", nz),
                                          ("Dxs", nx), ("Dys", ny), ("Dzs", nz))}
        self.L.ref_grid(*[p(m[k]) for k in ("X", "Y", "Z", "Dx", "Dy", "Dz", "Dxs", "Dys", "Dzs")])
        return m

    def eta(self):
        e = np.zeros(self.ng)
        self.L.ref_eta(p(e))
        return e

    def set_eta(self, e):
        self.L.ref_set_eta(p(e))

    def jp(self):
        a, b = np.zeros(self.n), np.zeros(self.n)
        self.L.ref_jp(p(a), p(b))
        return a, b

    def convdiff(self, u0, v0, w0, u1, v1, w1):
        self.L.ref_convdiff(p(u0), p(v0), p(w0), p(u1), p(v1), p(w1))

    def smagorinsky(self, u, v, w):
        """SmagorinskyModel of (u, v, w) (LES builds only); afterwards
        convdiff of the same T0 uses this eddy viscosity."""
        vis = np.zeros(self.n)
        self.L.ref_smagorinsky.argtypes = [_dp] * 4
        self.L.ref_smagorinsky(p(u), p(v), p(w), p(vis))
        return vis

    def rhs(self, kind, u1, v1, w1):
        b = np.zeros(self.n)
        self.L.ref_rhs(int(kind), p(u1), p(v1), p(w1), p(b))
        return b

    def spe_spmv(self, x):
        r = np.zeros(self.n)
        self.L.ref_spe_spmv(p(x), p(r))
        return r

    def ell_spmv(self, x):
        r = np.zeros(self.n)
        self.L.ref_ell_spmv(p(x), p(r))
        return r

    def bicg(self, kind, b, x):
        it, res = C.c_int(), C.c_double()
        self.L.ref_bicg(int(kind), p(b), p(x), C.byref(it), C.byref(res))
        return it.value, res.value

    def sor_seq(self, u1, v1, w1, pr, omega, tol, itmax):
        it, err = C.c_int(), C.c_double()
        self.L.ref_sor_seq(p(u1), p(v1), p(w1), p(pr), omega, tol, int(itmax), C.byref(it),
                           C.byref(err))
        return it.value, err.value

    def update_uf(self, pr, u1, v1, w1, u3, v3, w3, f):
        self.L.ref_update_uf(p(pr), p(u1), p(v1), p(w1), p(u3), p(v3), p(w3), p(f))

    def cdcl(self, f):
        cd, cl = C.c_double(), C.c_double()
        self.L.ref_cdcl(p(f), C.byref(cd), C.byref(cl))
        return cd.value, cl.value

    def bc_main(self, u, v, w, pr):
        self.L.ref_bc_main(p(u), p(v), p(w), p(pr))

    def bc_copy(self, uo, vo, wo, u, v, w):
        self.L.ref_bc_copy(p(uo), p(vo), p(wo), p(u), p(v), p(w))

    def pc_start(self, u0=None, v0=None, w0=None):
        self.L.ref_pc_start(p(u0), p(v0), p(w0))

    def pc_run(self, nsteps, method=0, solver=0, compat=False):
        cd, cl = np.zeros(nsteps), np.zeros(nsteps)
        it = np.zeros(4 * nsteps, dtype=np.int32)
        wall = np.zeros(nsteps)
        self.L.ref_pc_run(int(nsteps), int(method), int(solver), int(compat), p(cd), p(cl), p(it),
                          p(wall))
        return cd, cl, it.reshape(nsteps, 4), wall

    def state(self):
        u, v, w, pr = (np.zeros(self.ng) for _ in range(4))
        f, x = np.zeros(3 * self.n), np.zeros(self.n)
        self.L.ref_state(p(u), p(v), p(w), p(pr), p(f), p(x))
        return dict(u=u, v=v, w=w, p=pr, f=f, x=x)
