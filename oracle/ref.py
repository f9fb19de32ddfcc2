"""ctypes view of the reference oracle built by oracle/build_ref.py.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product.  Every call runs the
reference's own code (main.cu compiled for host cores); see ref_entry.cpp for
the list of wrapped functions and their main.cu lines.
"""
import ctypes
import os

import numpy as np

from . import build_ref

_cache = {}


def available():
    """True when the reference can be built here (checkout or extracted copy)."""
    return os.path.exists(os.path.join(build_ref.REF_DIR, "main.cu")) or os.path.exists(build_ref.GEN)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class RefOracle:
    def __init__(self, pl=31, opset=0, philox=0, project_math=1, rw_sd=0.0, map_delta=0.0):
        r = build_ref.build(pl, opset, philox, project_math, rw_sd, map_delta)
        if r is None:
            raise RuntimeError("reference source unavailable")
        self.so_path, self.cli_path = r
        self.lib = lib = ctypes.CDLL(self.so_path)
        self.PL = lib.gpr_ref_program_length()
        self.nops = lib.gpr_ref_nops()
        self.philox = bool(lib.gpr_ref_rng_is_philox())
        vp, ip, fp = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        lib.gpr_ref_run_kernel.argtypes = [ip, vp, vp, vp, ip, ip, vp, vp, ip, ip]
        lib.gpr_ref_run_kernel_range.argtypes = [ip, ip, ip, vp, vp, vp, ip, ip, vp, vp, ip, ip]
        lib.gpr_ref_prior.argtypes = [ip, ip, vp, vp]
        lib.gpr_ref_prior.restype = ctypes.c_double
        lib.gpr_ref_likelihood.argtypes = [ip, ip, vp, vp, vp, ip]
        lib.gpr_ref_likelihood.restype = ctypes.c_double
        lib.gpr_ref_count_nodes.argtypes = [ip, ip, vp, vp]
        lib.gpr_ref_length.argtypes = [ip, ip, vp, vp]
        lib.gpr_ref_length.restype = fp
        lib.gpr_ref_call.argtypes = [ip, ip, vp, vp, fp]
        lib.gpr_ref_call.restype = fp
        lib.gpr_ref_degree.argtypes = [ip, ip, vp, vp]
        lib.gpr_ref_degree.restype = fp
        lib.gpr_ref_display.argtypes = [ctypes.c_char_p, ip, ip, vp, vp, ip, ctypes.c_char_p, ip]
        lib.gpr_ref_opmap.argtypes = [ip]
        lib.gpr_ref_dev_random_int.argtypes = [ip, vp]
        lib.gpr_ref_dev_random_float.argtypes = [vp]
        lib.gpr_ref_dev_random_float.restype = fp
        lib.gpr_ref_dev_random_normal.argtypes = [vp]
        lib.gpr_ref_dev_random_normal.restype = fp
        lib.gpr_ref_dev_random_geometric.argtypes = [fp, vp]
        lib.gpr_ref_dev_random_geometric.restype = fp
        lib.gpr_ref_dev_seed.argtypes = [vp, ip, ip]
        lib.gpr_ref_dev_rand.argtypes = [vp]
        lib.gpr_ref_srand.argtypes = [ctypes.c_uint]
        lib.gpr_ref_host_random_int.argtypes = [ip]
        lib.gpr_ref_host_random_normal.restype = fp
        lib.gpr_ref_lnormalpdf.argtypes = [fp, fp]
        lib.gpr_ref_lnormalpdf.restype = ctypes.c_double
        lib.gpr_ref_lcauchypdf.argtypes = [fp, fp]
        lib.gpr_ref_lcauchypdf.restype = ctypes.c_double
        lib.gpr_ref_is_descendant.argtypes = [ip, ip]
        lib.gpr_ref_load_data.argtypes = [ctypes.c_char_p, fp, ip, ip, vp, ip]
        lib.gpr_ref_host_random_int.restype = ip
        lib.gpr_ref_host_init.argtypes = [vp, vp, ip, ctypes.c_uint]
        lib.gpr_ref_resample_cutoff.argtypes = [ip, vp, vp, vp]
        lib.gpr_ref_resample_cutoff.restype = ctypes.c_double
        self.ops = [lib.gpr_ref_opmap(k) for k in range(self.nops)]

    @staticmethod
    def pack_data(x, y, sd):
        d = np.empty((len(x), 3), np.float32)
        d[:, 0], d[:, 1], d[:, 2] = x, y, sd
        return np.ascontiguousarray(d)

    def run_kernel(self, P, C, x, y, sd, steps, seed, nthreads=0, chains=None):
        """One MH_simple_kernel block over all chains (or chains [c0, c1)).
        P (PL, N) int32 and C (PL, N) float32 are updated in place."""
        PL, N = P.shape
        assert PL == self.PL and P.dtype == np.int32 and C.dtype == np.float32
        assert P.flags.c_contiguous and C.flags.c_contiguous
        D = self.pack_data(x, y, sd)
        prior = np.zeros(N, np.float64)
        lik = np.zeros(N, np.float64)
        if chains is None:
            self.lib.gpr_ref_run_kernel(N, _p(P), _p(C), _p(D), len(x), steps, _p(prior), _p(lik),
                                        int(seed), nthreads)
        else:
            self.lib.gpr_ref_run_kernel_range(N, chains[0], chains[1], _p(P), _p(C), _p(D), len(x),
                                              steps, _p(prior), _p(lik), int(seed), nthreads)
        return prior, lik

    def prior(self, P, C, idx):
        return self.lib.gpr_ref_prior(P.shape[1], idx, _p(P), _p(C))

    def likelihood(self, P, C, idx, x, y, sd):
        D = self.pack_data(x, y, sd)
        return self.lib.gpr_ref_likelihood(P.shape[1], idx, _p(P), _p(C), _p(D), len(x))

    def count_nodes(self, P, C, idx):
        return self.lib.gpr_ref_count_nodes(P.shape[1], idx, _p(P), _p(C))

    def length(self, P, C, idx):
        return self.lib.gpr_ref_length(P.shape[1], idx, _p(P), _p(C))

    def call(self, P, C, idx, xv):
        return self.lib.gpr_ref_call(P.shape[1], idx, _p(P), _p(C), float(xv))

    def degree(self, P, C, idx):
        return self.lib.gpr_ref_degree(P.shape[1], idx, _p(P), _p(C))

    def display(self, fmt, P, C, idx, latex=False):
        n = self.lib.gpr_ref_display(fmt.encode(), P.shape[1], idx, _p(P), _p(C), int(latex), None, 0)
        buf = ctypes.create_string_buffer(n + 1)
        self.lib.gpr_ref_display(fmt.encode(), P.shape[1], idx, _p(P), _p(C), int(latex), buf, n + 1)
        return buf.value.decode("latin-1")


    def load_data(self, path, sdscale=1.0, first_half=False, even_half=False):
        out = np.empty((100000, 3), np.float32)
        n = self.lib.gpr_ref_load_data(path.encode(), sdscale, int(first_half), int(even_half), _p(out),
                                       out.shape[0])
        return out[:n, 0].copy(), out[:n, 1].copy(), out[:n, 2].copy()

    def resample_cutoff(self, prior, lik):
        """(cutoff, re-drawn flags) of main.cu:1215-1223 on these scores."""
        prior = np.ascontiguousarray(prior, np.float64)
        lik = np.ascontiguousarray(lik, np.float64)
        flags = np.zeros(len(prior), np.int32)
        cut = self.lib.gpr_ref_resample_cutoff(len(prior), _p(prior), _p(lik), _p(flags))
        return cut, flags.astype(bool)

    def host_init(self, N, seed):
        """srand(seed) then main.cu:1133-1137, with the reference's host RNG."""
        P = np.empty((self.PL, N), np.int32)
        C = np.empty((self.PL, N), np.float32)
        self.lib.gpr_ref_host_init(_p(P), _p(C), N, seed)
        return P, C


def get(**kw):
    key = tuple(sorted(kw.items()))
    if key not in _cache:
        _cache[key] = RefOracle(**kw)
    return _cache[key]
