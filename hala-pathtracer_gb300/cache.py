"""Stand-alone handle on the radiance cache (pt_cache_*): evaluation,
gradients and training on host arrays. The renderer owns its own cache
(Renderer.set_radiance_cache); this object exists for tests and tools.

Records are (n, 16) float32: position xyz, outgoing direction xyz, shading
normal xyz, base colour rgb, roughness, metallic, specular transmission, 0.
"""
import ctypes as C

import numpy as np

from . import PTError, _cache_config, abi, load_library


class RadianceCache:
    def __init__(self, **options):
        self._lib = load_library()
        self.config = _cache_config(**options)
        h = C.c_void_p()
        st = self._lib.pt_cache_create(C.byref(self.config), C.byref(h))
        if st != abi.PT_OK:
            raise PTError(st, "pt_cache_create failed")
        self._h = h
        m, g = C.c_uint64(), C.c_uint64()
        self._lib.pt_cache_num_params(self._h, C.byref(m), C.byref(g))
        self.n_mlp, self.n_grid = m.value, g.value

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pt_cache_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != abi.PT_OK:
            msg = self._lib.pt_cache_last_error(self._h)
            raise PTError(st, msg.decode() if msg else "")

    def set_bounds(self, lo, hi):
        self._check(self._lib.pt_cache_set_bounds(self._h, (C.c_float * 3)(*lo), (C.c_float * 3)(*hi)))

    def params(self):
        mlp = np.empty(self.n_mlp, np.float32)
        grid = np.empty(self.n_grid, np.float32)
        self._check(self._lib.pt_cache_get_params(self._h, mlp.ctypes.data, grid.ctypes.data))
        return mlp, grid

    def set_params(self, mlp=None, grid=None):
        m = None if mlp is None else np.ascontiguousarray(mlp, np.float32)
        g = None if grid is None else np.ascontiguousarray(grid, np.float32)
        self._check(self._lib.pt_cache_set_params(self._h, None if m is None else m.ctypes.data,
                                                  None if g is None else g.ctypes.data))

    def infer(self, records):
        r = np.ascontiguousarray(records, np.float32)
        out = np.empty((len(r), 3), np.float32)
        self._check(self._lib.pt_cache_infer(self._h, r.ctypes.data, len(r), out.ctypes.data))
        return out

    def gradients(self, records, targets):
        r = np.ascontiguousarray(records, np.float32)
        t = np.ascontiguousarray(targets, np.float32)
        gm = np.empty(self.n_mlp, np.float32)
        gg = np.empty(self.n_grid, np.float32)
        loss = C.c_float()
        self._check(self._lib.pt_cache_gradients(self._h, r.ctypes.data, t.ctypes.data, len(r), gm.ctypes.data,
                                                 gg.ctypes.data, C.byref(loss)))
        return gm, gg, loss.value

    def train(self, records, targets, steps=1):
        r = np.ascontiguousarray(records, np.float32)
        t = np.ascontiguousarray(targets, np.float32)
        loss = C.c_float()
        self._check(self._lib.pt_cache_train(self._h, r.ctypes.data, t.ctypes.data, len(r), int(steps),
                                             C.byref(loss)))
        return loss.value

    def benchmark(self, n=1 << 22, iterations=10):
        """Device ms of one inference and one training pass over n seeded records."""
        a, b = C.c_double(), C.c_double()
        self._check(self._lib.pt_cache_benchmark(self._h, int(n), int(iterations), C.byref(a), C.byref(b)))
        return a.value, b.value


def main(argv=None):
    """Device-timed cache kernels on seeded records (profiling entry point):
    python -m hala-pathtracer_gb300.cache --queries N --iterations K"""
    import argparse
    ap = argparse.ArgumentParser(description="radiance-cache kernel benchmark")
    ap.add_argument("--queries", type=int, default=1 << 22)
    ap.add_argument("--iterations", type=int, default=5)
    args = ap.parse_args(argv)
    c = RadianceCache()
    infer_ms, train_ms = c.benchmark(args.queries, args.iterations)
    c.close()
    print(f"{args.queries} records: inference {infer_ms:.3f} ms, training pass {train_ms:.3f} ms")
    return 0


if __name__ == "__main__":
    import sys
    sys.exit(main())
