"""Many independent realisations on one GPU through the batch entry points of the
C ABI (gic_batch_*): the whole realisation of every context (noise, linear
modifications, fields, particles) as one CUDA graph, each context on its own stream;
contexts with a variance modification from a pool of host threads beside it.

  gens = [ICGenerator(precision='mixed') for _ in range(64)]   # set up like any generator
  with Batch(gens) as b:
      b.realise(seeds=range(1, 65))                            # then gens[i].particles(l) ...
"""
import ctypes

from . import _lib


class Batch:
    def __init__(self, generators):
        self.generators = list(generators)
        self._lib = _lib.load()
        ctxs = (ctypes.c_void_p * len(self.generators))(*[g._ctx.value for g in self.generators])
        handle = ctypes.c_void_p()
        st = self._lib.gic_batch_create(ctypes.byref(handle), ctxs, len(self.generators))
        if st != _lib.GIC_OK:
            raise _lib.GicError(st, 'gic_batch_create failed: contexts must be distinct and on one device')
        self._handle = handle

    def realise(self, seeds, modes=None, order=1, threads=8):
        """One realisation of every generator: seeds[i] (and seeding modes[i], default
        the parallel Fourier mode), its queued modifications, then fields and particles."""
        seeds = list(seeds)
        n = len(self.generators)
        if len(seeds) != n:
            raise ValueError('one seed per generator')
        c_seeds = (ctypes.c_ulong * n)(*seeds)
        c_modes = (ctypes.c_int * n)(*modes) if modes is not None else None
        st = self._lib.gic_batch_realise(self._handle, c_seeds, c_modes, int(order), int(threads))
        if st != _lib.GIC_OK:
            raise _lib.GicError(st, self._lib.gic_batch_last_error(self._handle).decode())
        for g in self.generators:
            g._drawn = True

    def graph_info(self):
        """(contexts in the graph, kernels per replay, replays since capture, why
        capturing stopped or '')."""
        c, k, r, why = ctypes.c_int(), ctypes.c_ulonglong(), ctypes.c_int(), ctypes.c_char_p()
        self._lib.gic_batch_graph_info(self._handle, ctypes.byref(c), ctypes.byref(k), ctypes.byref(r),
                                       ctypes.byref(why))
        return c.value, k.value, r.value, (why.value or b'').decode()

    def stream(self):
        s = ctypes.c_void_p()
        self._lib.gic_batch_get_stream(self._handle, ctypes.byref(s))
        return s.value

    def close(self):
        if getattr(self, '_handle', None):
            self._lib.gic_batch_destroy(self._handle)
            self._handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
