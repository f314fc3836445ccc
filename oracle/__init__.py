"""Test infrastructure only: CPU checkers for the KDTree hot path.

Two interchangeable backends expose the same methods:

* ``"ref"``  -- the reference NBodylib KDTree compiled from its own sources
  (``oracle/_ref/libnbref.so``; buildable only where the reference checkout exists);
* ``"port"`` -- the C restatement in ``oracle/nbport.c`` (``oracle/_build/libnbport.so``),
  which builds anywhere and is pinned against ``"ref"`` and the golden fixtures.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may use
this package. Every per-particle array is in input order (the reference's particle ID).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libnbport.so")
REF_SO = os.path.join(HERE, "_ref", "libnbref.so")


def ref_src() -> str:
    """The reference checkout the "ref" backend compiles from: NBKDT_REF_SRC if set, else
    the REF default of oracle/Makefile (the build recipe is the one place that names it)."""
    env = os.environ.get("NBKDT_REF_SRC")
    if env:
        return env
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    return r.stdout.strip()


def ref_present(src: str | None = None) -> bool:
    src = src or ref_src()
    return bool(src) and os.path.isdir(os.path.join(src, "src", "KDTree"))

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)


def build(ref: bool = False, ref_src: str | None = None) -> None:
    """Compile the restatement (always) and the reference (if its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    src = ref_src or globals()["ref_src"]()
    if ref and ref_present(src):
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", f"REF={src}"], check=True)


def available(backend: str) -> bool:
    return os.path.exists(PORT_SO if backend == "port" else REF_SO)


_LIBS: dict[str, ctypes.CDLL] = {}


def _lib(backend: str) -> ctypes.CDLL:
    if backend in _LIBS:
        return _LIBS[backend]
    path = PORT_SO if backend == "port" else REF_SO
    if not os.path.exists(path):
        raise FileNotFoundError(f"oracle backend {backend!r} not built: {path}")
    lib = ctypes.CDLL(path)
    p = "pt_" if backend == "port" else "ref_"
    vp = ctypes.c_void_p
    sig = {
        "create": (vp, [_c_dbl_p, _c_dbl_p, _c_dbl_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                        ctypes.c_int, ctypes.c_int, _c_dbl_p, ctypes.c_int]),
        "destroy": (None, [vp]),
        "num_nodes": (ctypes.c_int, [vp]),
        "num_leaves": (ctypes.c_int, [vp]),
        "kernnorm": (ctypes.c_double, [vp]),
        "build_seconds": (ctypes.c_double, [vp]),
        "ids": (None, [vp, _c_int_p]),
        "leaf_start": (None, [vp, _c_int_p]),
        "knn": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _c_int_p, _c_dbl_p]),
        "veldensity": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, _c_dbl_p]),
        "density_particle": (ctypes.c_double, [vp, ctypes.c_int, ctypes.c_int]),
        "veldensity_particle": (ctypes.c_double, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
        "density_position": (ctypes.c_double, [vp, _c_dbl_p, ctypes.c_int]),
        "veldensity_position": (ctypes.c_double, [vp, _c_dbl_p, _c_dbl_p, ctypes.c_int,
                                                  ctypes.c_int]),
        "fof": (ctypes.c_int, [vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, _c_int_p, _c_int_p]),
        "fof_criterion": (ctypes.c_int, [vp, ctypes.c_int, _c_dbl_p, ctypes.c_int, ctypes.c_int,
                                         _c_int_p, _c_int_p]),
        "ball_tagged": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double, _c_int_p]),
        "ball_tagged_pos": (ctypes.c_int, [vp, _c_dbl_p, ctypes.c_double, _c_int_p]),
        "ball_mark": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, _c_int_p,
                                     _c_dbl_p]),
        "fof_nn": (ctypes.c_int, [vp, ctypes.c_int, _c_dbl_p, ctypes.c_int, _c_int_p, _c_dbl_p,
                                  ctypes.c_int, _c_int_p, ctypes.c_int, _c_int_p, _c_int_p]),
        "smooth_vel_moments": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, _c_dbl_p, _c_dbl_p,
                                              _c_dbl_p, _c_dbl_p]),
        "veldensity_phys": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, _c_dbl_p, _c_dbl_p]),
        "veldensity_phys_particle": (ctypes.c_double, [vp, ctypes.c_int, ctypes.c_int,
                                                       ctypes.c_int, _c_dbl_p]),
        "smooth_one": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, _c_dbl_p, ctypes.c_int,
                                      _c_dbl_p, _c_dbl_p, _c_dbl_p, ctypes.c_double, _c_dbl_p]),
    }
    if backend == "port":
        sig["set_aniso"] = (None, [vp, ctypes.c_int])
        sig["knn_coord"] = (ctypes.c_int, [vp, _c_dbl_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           _c_int_p, _c_dbl_p])
        sig["knn_pos"] = (ctypes.c_int, [vp, _c_dbl_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         _c_int_p, _c_dbl_p])
        sig["density"] = (ctypes.c_int, [vp, ctypes.c_int, _c_dbl_p, _c_int_p])
        sig["density_parallel"] = (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, _c_dbl_p])
        sig["veldensity_parallel"] = (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_int, _c_dbl_p])
        sig["kernel_table"] = (None, [vp, _c_dbl_p])
        sig["density_adjoint"] = (ctypes.c_int, [vp, ctypes.c_int, _c_int_p, _c_dbl_p, _c_dbl_p,
                                                 _c_dbl_p, _c_dbl_p, _c_dbl_p, _c_dbl_p])
        sig["density_frozen"] = (ctypes.c_int, [vp, ctypes.c_int, _c_int_p, _c_dbl_p, _c_dbl_p,
                                                _c_dbl_p, _c_dbl_p])
        sig["adj_create"] = (vp, [vp, ctypes.c_int, _c_int_p, _c_dbl_p, _c_dbl_p, _c_dbl_p])
        sig["adj_fd"] = (ctypes.c_double, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double])
        sig["adj_destroy"] = (None, [vp])
    else:
        sig["create_ex"] = (vp, sig["create"][1] + [ctypes.c_int])
        sig["knn_coord"] = (ctypes.c_int, [vp, _c_dbl_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           _c_int_p, _c_dbl_p])
        sig["knn_pos"] = (ctypes.c_int, [vp, _c_dbl_p, ctypes.c_int, ctypes.c_int, _c_int_p,
                                         _c_dbl_p])
        sig["density"] = (ctypes.c_int, [vp, ctypes.c_int, _c_dbl_p])
    for name, (res, args) in sig.items():
        f = getattr(lib, p + name)
        f.restype = res
        f.argtypes = args
    _LIBS[backend] = lib
    return lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(_c_dbl_p)


def _ip(a):
    return None if a is None else a.ctypes.data_as(_c_int_p)


class OracleTree:
    """A CPU kd-tree built by the reference (``ref``) or by the restatement (``port``)."""

    def __init__(self, pos, vel=None, mass=None, bucket_size=16, treetype=0, kerntype=0,
                 kernres=1000, period=None, backend="port", nthreads=0, aniso=0):
        self.backend = backend
        self._lib = _lib(backend)
        self._f = lambda name: getattr(self._lib, ("pt_" if backend == "port" else "ref_") + name)
        self.pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        self.n = self.pos.shape[0]
        self.vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
        self.mass = None if mass is None else np.ascontiguousarray(mass, dtype=np.float64)
        self.kernres = kernres
        per = None if period is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(period, dtype=np.float64), (3,)))
        self._per = per
        args = (_dp(self.pos), _dp(self.vel), _dp(self.mass), self.n, bucket_size, treetype,
                kerntype, kernres, _dp(per), nthreads)
        if backend == "port":
            self._h = self._f("create")(*args)
            self._f("set_aniso")(self._h, aniso)
        else:
            self._h = self._f("create_ex")(*args, aniso)
        self.treetype = treetype
        self.nd = 6 if treetype == 3 else 3
        self.nthreads = nthreads

    def close(self):
        if self._h:
            self._f("destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_nodes(self):
        return self._f("num_nodes")(self._h)

    @property
    def num_leaves(self):
        return self._f("num_leaves")(self._h)

    @property
    def kernnorm(self):
        return self._f("kernnorm")(self._h)

    @property
    def build_seconds(self):
        return self._f("build_seconds")(self._h)

    def ids(self):
        out = np.empty(self.n, np.int32)
        self._f("ids")(self._h, _ip(out))
        return out

    def leaf_start(self):
        out = np.empty(self.n, np.int32)
        self._f("leaf_start")(self._h, _ip(out))
        return out

    def kernel_table(self):
        out = np.empty(self.kernres, np.float64)
        self._f("kernel_table")(self._h, _dp(out))
        return out

    def knn(self, k, method=0):
        """method 0: FindNearest(tt); 1: FindNearestPos(tt). Rows by ID, neighbours as IDs."""
        nn = np.empty((self.n, k), np.int32)
        d2 = np.empty((self.n, k), np.float64)
        st = self._f("knn")(self._h, method, k, self.nthreads, _ip(nn), _dp(d2))
        if st:
            raise RuntimeError(f"FindNearest: status {st}")
        return nn, d2

    def knn_coord(self, x, k):
        """FindNearest(Double_t* x): x rows in the tree's space (3, or 6 for phase space)."""
        x = np.ascontiguousarray(x, np.float64).reshape(-1, self.nd)
        nn = np.empty((x.shape[0], k), np.int32)
        d2 = np.empty((x.shape[0], k), np.float64)
        if self.backend == "port":
            st = self._f("knn_coord")(self._h, _dp(x), x.shape[0], k, self.nthreads, _ip(nn),
                                      _dp(d2))
        else:
            st = self._f("knn_coord")(self._h, _dp(x), x.shape[0], self.nd, k, _ip(nn), _dp(d2))
        if st:
            raise RuntimeError(f"FindNearest(x): status {st}")
        return nn, d2

    def knn_pos(self, x, k):
        x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
        nn = np.empty((x.shape[0], k), np.int32)
        d2 = np.empty((x.shape[0], k), np.float64)
        if self.backend == "port":
            self._f("knn_pos")(self._h, _dp(x), x.shape[0], k, self.nthreads, _ip(nn), _dp(d2))
        else:
            self._f("knn_pos")(self._h, _dp(x), x.shape[0], k, _ip(nn), _dp(d2))
        return nn, d2

    def density(self, k, return_nn=False):
        rho = np.empty(self.n, np.float64)
        if self.backend == "port":
            nn = np.empty((self.n, k), np.int32) if return_nn else None
            st = self._f("density")(self._h, k, _dp(rho), _ip(nn))
            if st:
                raise RuntimeError(f"CalcDensity: status {st}")
            return (rho, nn) if return_nn else rho
        self._f("density")(self._h, k, _dp(rho))
        return rho

    # ---- SPH smoothing (KDCalcSmoothQuantities.cxx). rho=None: CalcDensity(nsmooth) first.
    def _arr(self, a, shape):
        return None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(shape)

    def smooth_vel_moments(self, which, nsmooth, rho=None, smvel=None, disp=None):
        """which 0: CalcSmoothVel (n,3); 1: CalcSmoothVelDisp (n,3,3); 2: Skew; 3: Kurtosis."""
        out = np.empty((self.n, 9 if which == 1 else 3), np.float64)
        st = self._f("smooth_vel_moments")(self._h, which, nsmooth,
                                           _dp(self._arr(rho, (self.n,))),
                                           _dp(self._arr(smvel, (self.n, 3))),
                                           _dp(self._arr(disp, (self.n, 9))), _dp(out))
        if st:
            raise RuntimeError("smoothing: fewer than nsmooth neighbours")
        return out.reshape(self.n, 3, 3) if which == 1 else out

    def veldensity_phys(self, nsmooth, nsearch, rho=None):
        out = np.empty(self.n, np.float64)
        st = self._f("veldensity_phys")(self._h, nsmooth, nsearch,
                                        _dp(self._arr(rho, (self.n,))), _dp(out))
        if st:
            raise RuntimeError("CalcVelDensityWithPhysDensity: fewer than nsearch neighbours")
        return out

    def veldensity_phys_particle(self, pid, nsmooth, nsearch, rho=None):
        return self._f("veldensity_phys_particle")(self._h, int(pid), nsmooth, nsearch,
                                                   _dp(self._arr(rho, (self.n,))))

    def smooth_one(self, which, nsmooth, pid=-1, x=None, rho=None, smvel=None, weight=None,
                   mean=0.0):
        """which 0: CalcSmoothVel{Particle,Position} (3); 1: ..VelDisp.. (3,3);
        4: CalcSmoothLocalMean{..}; 5: CalcSmoothLocalDisp{..}."""
        out = np.empty(9 if which == 1 else (3 if which == 0 else 1), np.float64)
        st = self._f("smooth_one")(self._h, which, int(pid), _dp(self._arr(x, (3,))), nsmooth,
                                   _dp(self._arr(rho, (self.n,))), _dp(self._arr(smvel, (3,))),
                                   _dp(self._arr(weight, (self.n,))), float(mean), _dp(out))
        if st:
            raise RuntimeError("smoothing: fewer than nsmooth neighbours")
        return out.reshape(3, 3) if which == 1 else (out if which == 0 else float(out[0]))

    def veldensity(self, nsmooth, nsearch):
        out = np.empty(self.n, np.float64)
        self._f("veldensity")(self._h, nsmooth, nsearch, _dp(out))
        return out

    def density_parallel(self, k, nthreads=0):
        """CalcDensity(k) with the searches over OpenMP threads (port only): each
        density differs from density()'s by the summation order of its terms."""
        rho = np.empty(self.n, np.float64)
        st = self._f("density_parallel")(self._h, k, nthreads, _dp(rho))
        if st:
            raise RuntimeError(f"CalcDensity (parallel): status {st}")
        return rho

    def veldensity_parallel(self, nsmooth, nsearch, nthreads=0):
        """CalcVelDensity over OpenMP threads (port only): bit-identical to veldensity()."""
        out = np.empty(self.n, np.float64)
        st = self._f("veldensity_parallel")(self._h, nsmooth, nsearch, nthreads, _dp(out))
        if st:
            raise RuntimeError(f"CalcVelDensity (parallel): status {st}")
        return out

    def density_particle(self, pid, k):
        return self._f("density_particle")(self._h, int(pid), k)

    def veldensity_particle(self, pid, nsmooth, nsearch):
        return self._f("veldensity_particle")(self._h, int(pid), nsmooth, nsearch)

    def density_position(self, x, k):
        """CalcDensityPosition(x, k) (physical or velocity tree; x in the tree's space)."""
        return self._f("density_position")(self._h, _dp(self._arr(x, (3,))), k)

    def veldensity_position(self, x, v, nsmooth, nsearch):
        """CalcVelDensityPosition(x, v, nsmooth, nsearch) (physical tree)."""
        return self._f("veldensity_position")(self._h, _dp(self._arr(x, (3,))),
                                              _dp(self._arr(v, (3,))), nsmooth, nsearch)

    def fof(self, ll, minnum=8, order=0):
        g = np.empty(self.n, np.int32)
        ng = ctypes.c_int(0)
        self._f("fof")(self._h, float(ll), minnum, order, _ip(g), ctypes.byref(ng))
        return g, ng.value

    def fof_criterion(self, cmp, params, minnum=8, order=0):
        p = np.zeros(20, np.float64)
        p[: len(params)] = params
        g = np.empty(self.n, np.int32)
        ng = ctypes.c_int(0)
        self._f("fof_criterion")(self._h, cmp, _dp(p), minnum, order, _ip(g), ctypes.byref(ng))
        return g, ng.value

    def fof_nn(self, cmp, params, nn, minnum=8, values=None, pidx=None, dist2=None):
        """FOFNNCriterion over lists nn (rows by this tree's index, tree indices). The
        restatement takes per-target values (tree order) with parameter indices pidx; the
        reference takes the lists' dist2 and uses the row maximum as its distfunc."""
        p = np.zeros(20)
        p[:len(params)] = params
        nn = np.ascontiguousarray(nn, np.int32)
        numnn = nn.shape[1]
        group = np.empty(self.n, np.int32)
        ng = ctypes.c_int()
        pi = None if pidx is None else np.ascontiguousarray(pidx, np.int32)
        npc = 0 if pi is None else len(pi)
        if self.backend == "port":
            vals = None if values is None else np.ascontiguousarray(values, np.float64)
            self._f("fof_nn")(self._h, cmp, _dp(p), numnn, _ip(nn), _dp(vals), npc, _ip(pi),
                              minnum, _ip(group), ctypes.byref(ng))
        else:
            d2 = None if dist2 is None else np.ascontiguousarray(dist2, np.float64)
            self._f("fof_nn")(self._h, cmp, _dp(p), numnn, _ip(nn), _dp(d2), npc, _ip(pi),
                              minnum, _ip(group), ctypes.byref(ng))
        return group, ng.value

    def tree_knn(self, k):
        """FindNearest rows by this tree's index holding tree indices (the lists
        FOFNNCriterion takes), with their d2."""
        nn, d2 = self.knn(k, method=0)  # rows by ID, IDs
        ids = self.ids()  # tree index -> ID
        tree_of = np.empty_like(ids)
        tree_of[ids] = np.arange(len(ids))
        return (np.ascontiguousarray(tree_of[nn[ids]], np.int32),
                np.ascontiguousarray(d2[ids]))

    def ball_tagged(self, pid, fdist2):
        out = np.empty(8 * self.n + 16, np.int32)
        c = self._f("ball_tagged")(self._h, int(pid), float(fdist2), _ip(out))
        return np.sort(out[:c])

    def ball_tagged_pos(self, x, fdist2):
        x = np.ascontiguousarray(x, np.float64).reshape(3)
        out = np.empty(8 * self.n + 16, np.int32)
        c = self._f("ball_tagged_pos")(self._h, _dp(x), float(fdist2), _ip(out))
        return np.sort(out[:c])

    def ball_mark(self, pid, fdist2, imark=1):
        mark = np.zeros(self.n, np.int32)
        d2 = np.zeros(self.n, np.float64)
        self._f("ball_mark")(self._h, int(pid), float(fdist2), imark, _ip(mark), _dp(d2))
        return mark, d2

    def density_adjoint(self, k, nn_ids, weights, pos=None, mass=None):
        pos = self.pos if pos is None else np.ascontiguousarray(pos, np.float64)
        mass = self.mass if mass is None else np.ascontiguousarray(mass, np.float64)
        nn_ids = np.ascontiguousarray(nn_ids, np.int32)
        w = np.ascontiguousarray(weights, np.float64)
        rho = np.empty(self.n)
        gp = np.empty((self.n, 3))
        gm = np.empty(self.n)
        self._f("density_adjoint")(self._h, k, _ip(nn_ids), _dp(pos), _dp(mass), _dp(w), _dp(rho),
                                   _dp(gp), _dp(gm))
        return rho, gp, gm

    def local_fd(self, k, nn_ids, weights, coords, step=1e-6, mass=None):
        """Central finite differences dL/dpos[a, d] for every (a, d) in coords, on the
        frozen model, differencing only the affected loss terms."""
        mass = self.mass if mass is None else np.ascontiguousarray(mass, np.float64)
        nn_ids = np.ascontiguousarray(nn_ids, np.int32)
        w = np.ascontiguousarray(weights, np.float64)
        ctx = self._f("adj_create")(self._h, k, _ip(nn_ids), _dp(self.pos), _dp(mass), _dp(w))
        try:
            return np.array([self._f("adj_fd")(ctx, int(a), int(d), float(step))
                             for a, d in coords])
        finally:
            self._f("adj_destroy")(ctx)

    def density_frozen(self, k, nn_ids, pos0, pos, mass=None):
        mass = self.mass if mass is None else np.ascontiguousarray(mass, np.float64)
        rho = np.empty(self.n)
        self._f("density_frozen")(self._h, k, _ip(np.ascontiguousarray(nn_ids, np.int32)),
                                  _dp(np.ascontiguousarray(pos0, np.float64)),
                                  _dp(np.ascontiguousarray(pos, np.float64)), _dp(mass), _dp(rho))
        return rho
