"""ctypes binding of libgicgpu.so (include/gicgpu.h).

The CUDA library is the only implementation of the field-realisation path: if
it is missing, loading fails loudly instead of falling back to anything else.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, 'libgicgpu.so')

GIC_OK = 0
GIC_ERR_INVALID_ARG = -1
GIC_ERR_OOM = -2
GIC_ERR_CUDA = -3
GIC_ERR_TIMEOUT = -4
GIC_ERR_NOT_READY = -5
GIC_ERR_INTERNAL = -6

GIC_FP64 = 0
GIC_MIXED = 1

GIC_SEED_REAL_SPACE = 0
GIC_SEED_FOURIER_SERIAL = 1
GIC_SEED_FOURIER_PARALLEL = 2
GIC_SEED_FOURIER_REVERSE = 3

GIC_MOD_OVERDENSITY = 0
GIC_MOD_VX = 1
GIC_MOD_VY = 2
GIC_MOD_VZ = 3
GIC_MOD_POTENTIAL = 4
GIC_MOD_LX = 5
GIC_MOD_LY = 6
GIC_MOD_LZ = 7

GIC_FIELD_NOISE = 0
GIC_FIELD_DELTA = 1
GIC_FIELD_PSI_X = 2
GIC_FIELD_PSI_Y = 3
GIC_FIELD_PSI_Z = 4
GIC_NOISE_REVERSE = 0
GIC_NOISE_REVERSE_SMALL_K = 1
GIC_NOISE_UNIT_MODULUS = 2
GIC_FIELD_PSI2_X = 5
GIC_FIELD_PSI2_Y = 6
GIC_FIELD_PSI2_Z = 7


class GicDeviceOpts(ctypes.Structure):
    _fields_ = [('precision', ctypes.c_int), ('device', ctypes.c_int), ('mem_limit', ctypes.c_size_t)]


class GicCosmo(ctypes.Structure):
    _fields_ = [(name, ctypes.c_double) for name in
                ('omega_m', 'omega_lambda', 'omega_b', 'hubble', 'sigma8', 'ns', 'redshift')]


_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.c_int


GIC_MAP_MAX_LEVELS = 8


class GicParticleMap(ctypes.Structure):
    """gic_particle_map: the particles of a multi-level context in genetIC's mapper order."""
    _fields_ = [('nlevels', ctypes.c_int), ('n', ctypes.c_int * GIC_MAP_MAX_LEVELS),
                ('ratio', ctypes.c_int * GIC_MAP_MAX_LEVELS), ('origin', (ctypes.c_int * 3) * GIC_MAP_MAX_LEVELS),
                ('replaced', ctypes.POINTER(ctypes.c_ulonglong) * GIC_MAP_MAX_LEVELS),
                ('n_replaced', ctypes.c_ulonglong * GIC_MAP_MAX_LEVELS),
                ('mass', ctypes.c_double * GIC_MAP_MAX_LEVELS), ('eps', ctypes.c_double * GIC_MAP_MAX_LEVELS),
                ('pos_factor', ctypes.c_double), ('vel_factor', ctypes.c_double), ('mass_factor', ctypes.c_double)]

    @classmethod
    def of(cls, levels, replaced, mass, eps, pos_factor, vel_factor, mass_factor):
        """levels: [(n, ratio, (ox, oy, oz))] (ratio and origin unused on level 0);
        replaced: one array of ascending cell ids per level (the finest empty)."""
        import numpy as np
        m = cls()
        m.nlevels = len(levels)
        m._keep = []
        for l, (n, ratio, origin) in enumerate(levels):
            m.n[l] = n
            m.ratio[l] = ratio
            for a in range(3):
                m.origin[l][a] = origin[a]
            rep = np.ascontiguousarray(replaced[l] if l < len(replaced) else [], dtype=np.uint64)
            m._keep.append(rep)
            m.replaced[l] = rep.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong))
            m.n_replaced[l] = len(rep)
            m.mass[l] = mass[l]
            m.eps[l] = eps[l]
        m.pos_factor, m.vel_factor, m.mass_factor = pos_factor, vel_factor, mass_factor
        return m
# symbol -> argument types (all return int unless noted)
SIGNATURES = {
    'gic_create': [ctypes.POINTER(_P), ctypes.POINTER(GicDeviceOpts)],
    'gic_destroy': [_P],
    'gic_last_error': [_P],
    'gic_level_add': [_P, ctypes.c_double, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                      ctypes.POINTER(_I)],
    'gic_set_cosmology': [_P, ctypes.POINTER(GicCosmo)],
    'gic_set_transfer': [_P, _D, _I, _I],
    'gic_get_normalisation': [_P, _D, _D],
    'gic_draw_noise': [_P, ctypes.c_ulong, _I],
    'gic_gaussian_stream': [_P, ctypes.c_ulong, ctypes.c_size_t, _D],
    'gic_gaussian_stream_noalloc': [ctypes.c_ulong, ctypes.c_size_t, _P, _P],
    'gic_fetch_particles_native': [_P, _I, _D, _P],
    'gic_fetch_particles_resampled': [_P, _I, _I, _D, _D],
    'gic_fetch_particles_matched': [_P, _I, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_size_t, _D, _D],
    'gic_memory_use': [_P, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)],
    'gic_set_fft_wait': [_P, ctypes.c_uint, _I],
    'gic_set_noise': [_P, _I, _D],
    'gic_zeldovich': [_P, _I],
    'gic_fetch_level': [_P, _I, _I, _D],
    'gic_fetch_particles': [_P, _I, _D, _D],
    'gic_fft': [_P, _I, _I, _I],
    'gic_fft_box': [_P, _I, _I, _I, _P, _P],
    'gic_chi2': [_P, _D],
    'gic_launch_count': [ctypes.POINTER(ctypes.c_ulonglong)],
    'gic_calculate': [_P, _I, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_size_t, _D],
    'gic_add_modification': [_P, _I, ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_size_t, ctypes.c_double, _I],
    'gic_clear_modifications': [_P],
    'gic_noise_op': [_P, _I, ctypes.c_double],
    'gic_splice': [_P, ctypes.c_ulong, ctypes.POINTER(_P), ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(_I)],
    'gic_fetch_particles_async': [_P, _I, _D, _P],
    'gic_fetch_wait': [_P],
    'gic_grafic_pack': [_P, _P, _I, _I, _P, _P, _P, _P],
    'gic_fft_choice': [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)],
    'gic_batch_create': [ctypes.POINTER(_P), ctypes.POINTER(_P), _I],
    'gic_batch_destroy': [_P],
    'gic_batch_realise': [_P, ctypes.POINTER(ctypes.c_ulong), ctypes.POINTER(_I), _I, _I],
    'gic_batch_last_error': [_P],
    'gic_batch_get_stream': [_P, ctypes.POINTER(_P)],
    'gic_batch_graph_info': [_P, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(_I),
                             ctypes.POINTER(ctypes.c_char_p)],
    'gic_noise_real': [_P, _I, _P],
    'gic_field_from_noise': [_P, _I, _I, ctypes.POINTER(_P), _P],
    'gic_field_from_noise_adjoint': [_P, _I, _I, _P, ctypes.POINTER(_P)],
    'gic_variance_gradient': [_P, ctypes.POINTER(_P), ctypes.POINTER(ctypes.c_size_t), ctypes.c_double,
                              ctypes.POINTER(_P), ctypes.POINTER(_P), _I, _D],
    'gic_calculate_variance': [_P, ctypes.POINTER(_P), ctypes.POINTER(ctypes.c_size_t), ctypes.c_double, _D],
    'gic_add_variance_modification': [_P, ctypes.POINTER(_P), ctypes.POINTER(ctypes.c_size_t), ctypes.c_double,
                                      ctypes.c_double, _I, _I, ctypes.c_double],
    'gic_apply_modifications': [_P, _D, _D],
    'gic_get_stream': [_P, ctypes.POINTER(_P)],
    'gic_tipsy_count': [_P, ctypes.POINTER(ctypes.c_ulonglong)],
    'gic_tipsy_factors': [_P, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, _D, _D, _D],
    'gic_tipsy_pack_host': [_P, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.c_ulonglong, ctypes.c_ulonglong, _P, _I],
    'gic_tipsy_pack': [_P, _P, ctypes.c_ulonglong, ctypes.c_ulonglong, _P],
    'gic_tipsy_pack_async': [_P, _P, ctypes.c_ulonglong, ctypes.c_ulonglong, _P],
    'gic_gadget_pack': [_P, _P, ctypes.POINTER(_I), ctypes.c_ulonglong, ctypes.c_ulonglong, _P, _P, _P, _P],
    'gic_gadget_pack_host': [_P, ctypes.POINTER(_D), ctypes.POINTER(_D), ctypes.POINTER(_I), ctypes.c_ulonglong,
                             ctypes.c_ulonglong, _P, _P, _P, _P, _I],
}

_lib = None


def load():
    """Load libgicgpu.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError('libgicgpu.so is not built (run genetic_gb300/build.py): %s' % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_char_p if name in ('gic_last_error', 'gic_batch_last_error') else ctypes.c_int
    _lib = lib
    return lib


class GraficGrid(ctypes.Structure):
    """gic_grafic_grid: one grid of genetIC's grafic stack (include/gicgpu.h)."""
    _fields_ = [('level', ctypes.c_int), ('factor', ctypes.c_int), ('roll', ctypes.c_int * 3),
                ('vel_factor', ctypes.c_double), ('pos_factor', ctypes.c_double), ('id_offset', ctypes.c_ulonglong)]


class GicError(RuntimeError):
    def __init__(self, code, message):
        super().__init__('%s (status %d)' % (message, code))
        self.code = code


def check(ctx, status):
    if status != GIC_OK:
        msg = load().gic_last_error(ctx)
        raise GicError(status, msg.decode() if msg else 'error')
