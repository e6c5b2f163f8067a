"""ctypes binding of libmcwalk.so (declarations in include/mcwalk.h).

The library is the only compute path: if it is missing or no CUDA device is
present, these functions raise instead of falling back to anything else.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, '_lib', 'libmcwalk.so')

MCW_OK = 0
ABI_VERSION = 3          # MCW_ABI_VERSION of include/mcwalk.h these bindings follow
ERRORS = {-1: 'MCW_ERR_ARG', -2: 'MCW_ERR_CUDA', -3: 'MCW_ERR_BUDGET', -4: 'MCW_ERR_STREAM',
          -5: 'MCW_ERR_OOM', -6: 'MCW_ERR_STATE'}
MODE_F32 = 0
MODE_REPLAY64 = 1
MODE_POL64 = 2
MODE_POL32 = 3
RECORDS_NONE, RECORDS_HOST, RECORDS_DEVICE = 0, 1, 2
HIST_NTHETA, HIST_NPHI, HIST_BINS = 18, 36, 648
WVN_FX_SCALE = 4294967296.0
NOALLOC_MAX_LUT = 2048       # MCW_NOALLOC_MAX_LUT: wavelength grid points of mcw_walk_noalloc
DEFAULT_BUDGET_S = 300.0     # MCW_DEFAULT_BUDGET_S: time budget of a new context

# names every build of the library must export (the entry points of mcwalk.h)
EXPORTS = ['mcw_abi_version', 'mcw_version', 'mcw_create', 'mcw_destroy', 'mcw_last_error',
           'mcw_set_tables', 'mcw_set_launch', 'mcw_get_launch', 'mcw_set_budget', 'mcw_walk',
           'mcw_brf', 'mcw_autotune', 'mcw_graph_create', 'mcw_graph_launch',
           'mcw_graph_destroy', 'mcw_host_alloc', 'mcw_host_free', 'mcw_write_csv',
           'mcw_format_csv', 'mcw_walk_noalloc', 'mcw_post', 'mcw_set_phase_matrices']


class McwError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__('%s (%d): %s' % (ERRORS.get(code, 'MCW_ERR'), code, msg))
        self.code = code


class BudgetExceeded(McwError):
    pass


class SSPTableC(ctypes.Structure):
    _fields_ = [('wvl', ctypes.c_void_p), ('ss_alb', ctypes.c_void_p),
                ('ext_cff_mss', ctypes.c_void_p), ('asm_prm', ctypes.c_void_p),
                ('n', ctypes.c_int32), ('wvl_unit', ctypes.c_int32)]


class ConfigC(ctypes.Structure):
    _fields_ = [('n_photon', ctypes.c_int64), ('first_photon', ctypes.c_int64),
                ('wvl0', ctypes.c_double),
                ('half_width', ctypes.c_double), ('theta0_deg', ctypes.c_double),
                ('tau_tot', ctypes.c_double), ('imp_cnc', ctypes.c_double),
                ('rho_snw', ctypes.c_double), ('rho_ice', ctypes.c_double),
                ('lambertian_reflectance', ctypes.c_double),
                ('lambertian_surface', ctypes.c_int32), ('lambertian_bottom', ctypes.c_int32),
                ('ice_table', ctypes.c_int32), ('ssp_nearest', ctypes.c_int32),
                ('ssa_ice_override', ctypes.c_double), ('g_override', ctypes.c_double),
                ('ext_ice_override', ctypes.c_double), ('ssa_imp_override', ctypes.c_double),
                ('ext_imp_override', ctypes.c_double),
                ('polarised', ctypes.c_int32), ('pad', ctypes.c_int32),
                ('stokes0', ctypes.c_double * 4)]


class PhaseTableC(ctypes.Structure):
    _fields_ = [('n_rows', ctypes.c_int32), ('n_angle', ctypes.c_int32 * 6), ('pad', ctypes.c_int32),
                ('cos_asc', ctypes.c_void_p * 6), ('p_asc', ctypes.c_void_p * 6),
                ('a1', ctypes.c_void_p), ('a2', ctypes.c_void_p), ('b1', ctypes.c_void_p),
                ('b2', ctypes.c_void_p), ('cos_max', ctypes.c_double), ('cos_min', ctypes.c_double),
                ('cos_cutoff', ctypes.c_double)]


class StatsC(ctypes.Structure):
    _fields_ = [('kernel_ms', ctypes.c_double), ('total_ms', ctypes.c_double),
                ('device_ms', ctypes.c_double), ('h2d_bytes', ctypes.c_uint64),
                ('d2h_bytes', ctypes.c_uint64),
                ('n_photon', ctypes.c_uint64), ('n_events', ctypes.c_uint64),
                ('max_n_scat', ctypes.c_uint32), ('status', ctypes.c_uint32),
                ('block_size', ctypes.c_int32), ('blocks_per_sm', ctypes.c_int32),
                ('regen_chunk', ctypes.c_int32), ('grid', ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LaunchC(ctypes.Structure):
    _fields_ = [('block_size', ctypes.c_int32), ('blocks_per_sm', ctypes.c_int32),
                ('regen_chunk', ctypes.c_int32), ('drain_from', ctypes.c_int32)]


class GemmC(ctypes.Structure):
    """McwGemm of include/mcw_mlp.h."""
    _fields_ = [('m', ctypes.c_int32), ('n', ctypes.c_int32), ('k', ctypes.c_int32),
                ('trans_a', ctypes.c_int32), ('trans_b', ctypes.c_int32),
                ('epilogue', ctypes.c_int32), ('a', ctypes.c_void_p), ('lda', ctypes.c_int32),
                ('ldb', ctypes.c_int32), ('b', ctypes.c_void_p), ('bias', ctypes.c_void_p),
                ('aux', ctypes.c_void_p), ('ldaux', ctypes.c_int32), ('ldc', ctypes.c_int32),
                ('c', ctypes.c_void_p), ('c2', ctypes.c_void_p), ('ldc2', ctypes.c_int32),
                ('engine', ctypes.c_int32)]


class GemmGroupedC(ctypes.Structure):
    """McwGemmGrouped of include/mcw_mlp.h."""
    _fields_ = [('m', ctypes.c_int32), ('n', ctypes.c_int32), ('k', ctypes.c_int32),
                ('groups', ctypes.c_int32), ('splits', ctypes.c_int32), ('epilogue', ctypes.c_int32),
                ('a', ctypes.c_void_p), ('lda', ctypes.c_int64), ('stride_a', ctypes.c_int64),
                ('b', ctypes.c_void_p), ('ldb', ctypes.c_int64), ('stride_b', ctypes.c_int64),
                ('bias', ctypes.c_void_p), ('stride_bias', ctypes.c_int64),
                ('aux', ctypes.c_void_p), ('ldaux', ctypes.c_int64), ('stride_aux', ctypes.c_int64),
                ('c', ctypes.c_void_p), ('ldc', ctypes.c_int64), ('stride_c', ctypes.c_int64),
                ('stride_split', ctypes.c_int64),
                ('c2', ctypes.c_void_p), ('ldc2', ctypes.c_int64), ('stride_c2', ctypes.c_int64),
                ('ct', ctypes.c_void_p), ('ldct', ctypes.c_int64), ('stride_ct', ctypes.c_int64)]


class ColsumLayerC(ctypes.Structure):
    """McwColsumLayer of include/mcw_mlp.h."""
    _fields_ = [('g', ctypes.c_void_p), ('ld', ctypes.c_int64), ('stride', ctypes.c_int64),
                ('out_offset', ctypes.c_int64), ('n', ctypes.c_int32), ('pad', ctypes.c_int32)]


class TransposeBlockC(ctypes.Structure):
    """McwTransposeBlock of include/mcw_mlp.h."""
    _fields_ = [('offset', ctypes.c_int64), ('offset_t', ctypes.c_int64), ('ld_t', ctypes.c_int64),
                ('rows', ctypes.c_int32), ('cols', ctypes.c_int32)]


EPI_F32, EPI_BIAS_F32, EPI_BIAS_SILU, EPI_DSILU = 0, 1, 2, 3
ENGINE_MMA_SYNC, ENGINE_TCGEN05 = 0, 1

# entry points of include/mcw_mlp.h
MLP_EXPORTS = ['mcw_mlp_gemm', 'mcw_mlp_colsum', 'mcw_mlp_loss', 'mcw_mlp_adam', 'mcw_mlp_cast_bf16',
               'mcw_mlp_status', 'mcw_mlp_pack', 'mcw_mlp_forward', 'mcw_mlp_forward_f16',
               'mcw_mlp_forward_ensemble_f16',
               'mcw_mlp_gemm_grouped', 'mcw_mlp_reduce_splits', 'mcw_mlp_loss_grouped',
               'mcw_mlp_colsum_grouped', 'mcw_mlp_adam_grouped', 'mcw_mlp_gather', 'mcw_mlp_advance']
MLP_PACK_BYTES = 5 * 256 * 256 * 2 + 256 * 16 * 2
MLP_BIAS_FLOATS = 3 * 256 + 649

RECORD32 = np.dtype([('condition', np.int32), ('n_scat', np.int32), ('wvn', np.float32),
                     ('theta_n', np.float32), ('phi_n', np.float32),
                     ('path_length', np.float32), ('snow_depth', np.float32),
                     ('config', np.uint32)])
RECORD64 = np.dtype([('condition', np.int32), ('n_scat', np.int32), ('wvn', np.float64),
                     ('theta_n', np.float64), ('phi_n', np.float64),
                     ('path_length', np.float64), ('snow_depth', np.float64),
                     ('config', np.uint32), ('flags', np.uint32)])
RECORD64P = np.dtype([('condition', np.int32), ('n_scat', np.int32), ('wvn', np.float64),
                      ('theta_n', np.float64), ('phi_n', np.float64),
                      ('path_length', np.float64), ('snow_depth', np.float64),
                      ('config', np.uint32), ('flags', np.uint32),
                      ('stokes_q', np.float64), ('stokes_u', np.float64), ('stokes_v', np.float64)])
RECORD32P = np.dtype([('condition', np.int32), ('n_scat', np.int32), ('wvn', np.float32),
                      ('theta_n', np.float32), ('phi_n', np.float32),
                      ('path_length', np.float32), ('snow_depth', np.float32),
                      ('config', np.uint32), ('stokes_q', np.float32), ('stokes_u', np.float32),
                      ('stokes_v', np.float32), ('pad', np.float32)])
TALLY = np.dtype([('n_cond', np.uint64, 6), ('q_cond_fx', np.uint64, 6), ('n_events', np.uint64),
                  ('max_n_scat', np.uint32), ('reserved', np.uint32),
                  ('bin_wvn_fx', np.uint64, HIST_BINS), ('bin_count', np.uint32, HIST_BINS)])
POST_STATS = np.dtype([('q_cond_fx', np.uint64, 6), ('n_cond', np.uint64, 6), ('sum_n_scat', np.uint64),
                       ('sum_path_length', np.float64), ('sum_wavelength', np.float64)])
assert RECORD32.itemsize == 32 and RECORD64.itemsize == 56 and RECORD64P.itemsize == 80
assert RECORD32P.itemsize == 48
assert ctypes.sizeof(ConfigC) == 176 and ctypes.sizeof(StatsC) == 80

_lib = None


def load(path=None):
    """Load libmcwalk.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError('libmcwalk.so is not built (%s); run '
                           '`python -m monte_carlompi_gb300.build`' % p)
    L = ctypes.CDLL(p)
    vp, i32, i64, u64, dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double
    sig = {
        'mcw_abi_version': ([], ctypes.c_int),
        'mcw_version': ([], ctypes.c_char_p),
        'mcw_create': ([ctypes.c_int, ctypes.POINTER(vp)], ctypes.c_int),
        'mcw_destroy': ([vp], ctypes.c_int),
        'mcw_last_error': ([vp, ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
        'mcw_set_tables': ([vp, ctypes.POINTER(SSPTableC), i32, ctypes.POINTER(SSPTableC)], ctypes.c_int),
        'mcw_set_phase_matrices': ([vp, ctypes.POINTER(PhaseTableC), i32], ctypes.c_int),
        'mcw_set_launch': ([vp, ctypes.POINTER(LaunchC)], ctypes.c_int),
        'mcw_get_launch': ([vp, ctypes.POINTER(LaunchC)], ctypes.c_int),
        'mcw_set_budget': ([vp, dbl], ctypes.c_int),
        'mcw_walk': ([vp, ctypes.POINTER(ConfigC), i32, u64, i32, vp, i32, vp,
                      ctypes.POINTER(StatsC)], ctypes.c_int),
        'mcw_brf': ([vp, i32, vp, vp], ctypes.c_int),
        'mcw_autotune': ([vp, ctypes.POINTER(ConfigC), i32, u64, ctypes.POINTER(LaunchC),
                          ctypes.POINTER(dbl)], ctypes.c_int),
        'mcw_graph_create': ([vp, ctypes.POINTER(ConfigC), i32, vp, ctypes.POINTER(vp)], ctypes.c_int),
        'mcw_graph_launch': ([vp, u64, vp, ctypes.POINTER(StatsC)], ctypes.c_int),
        'mcw_graph_destroy': ([vp], ctypes.c_int),
        'mcw_host_alloc': ([ctypes.c_size_t, ctypes.POINTER(vp)], ctypes.c_int),
        'mcw_host_free': ([vp], ctypes.c_int),
        'mcw_write_csv': ([ctypes.c_char_p, vp, i32, i64, i32], ctypes.c_int),
        'mcw_format_csv': ([vp, i32, i64, i32, vp, ctypes.c_size_t,
                            ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
        'mcw_walk_noalloc': ([ctypes.POINTER(ConfigC), ctypes.POINTER(SSPTableC),
                              ctypes.POINTER(SSPTableC), u64, vp, vp, vp], ctypes.c_int),
        'mcw_post': ([vp, vp, i32, i32, i64, i32, i32, vp, vp, vp], ctypes.c_int),
        'mcw_mlp_gemm': ([ctypes.POINTER(GemmC), vp], ctypes.c_int),
        'mcw_mlp_colsum': ([vp, i32, i32, i32, vp, vp], ctypes.c_int),
        'mcw_mlp_loss': ([vp, i32, vp, i32, vp, i32, i32, vp, i32, vp, i32, vp, vp], ctypes.c_int),
        'mcw_mlp_adam': ([vp, vp, vp, vp, vp, i64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, i64, vp], ctypes.c_int),
        'mcw_mlp_cast_bf16': ([vp, vp, i64, vp], ctypes.c_int),
        'mcw_mlp_status': ([i32, ctypes.POINTER(ctypes.c_uint32)], ctypes.c_int),
        'mcw_mlp_pack': ([vp, vp, vp, vp, vp, vp], ctypes.c_int),
        'mcw_mlp_forward': ([vp, i32, vp, vp, vp, vp, vp, vp, i32, vp], ctypes.c_int),
        'mcw_mlp_forward_f16': ([vp, i32, vp, vp, vp, vp, vp, vp, i32, vp], ctypes.c_int),
        'mcw_mlp_forward_ensemble_f16': ([vp, i32, i32, vp, vp, vp, i32, vp], ctypes.c_int),
        'mcw_mlp_gemm_grouped': ([ctypes.POINTER(GemmGroupedC), vp], ctypes.c_int),
        'mcw_mlp_reduce_splits': ([vp, i64, i64, i64, vp, i64, i64, i32, i32, i32, i32, vp], ctypes.c_int),
        'mcw_mlp_loss_grouped': ([vp, i64, i64, vp, i64, i64, vp, i32, i32, i32, vp, i64, i64, vp, i64,
                                  vp, i64, i64, vp, vp], ctypes.c_int),
        'mcw_mlp_colsum_grouped': ([ctypes.POINTER(ColsumLayerC), i32, i32, i32, vp, i64, vp, i32, vp],
                                   ctypes.c_int),
        'mcw_mlp_adam_grouped': ([vp, vp, vp, vp, vp, i64, i32, vp, vp, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float, vp, i64, ctypes.POINTER(TransposeBlockC), i32, vp],
                                 ctypes.c_int),
        'mcw_mlp_gather': ([vp, vp, i64, i32, vp, i64, vp, i32, i32, vp, i64, vp, i64, vp, i64, i64, vp],
                           ctypes.c_int),
        'mcw_mlp_advance': ([vp, vp, vp], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    if L.mcw_abi_version() != ABI_VERSION:
        raise RuntimeError('%s has ABI version %d, these bindings need %d; rebuild it with '
                           '`python -m monte_carlompi_gb300.build`' % (p, L.mcw_abi_version(), ABI_VERSION))
    if path is None:
        _lib = L
    return L


def last_error(ctx):
    buf = ctypes.create_string_buffer(512)
    load().mcw_last_error(ctx, buf, 512)
    return buf.value.decode(errors='replace')


def check(rc, ctx=None, what=''):
    if rc == MCW_OK:
        return
    msg = last_error(ctx) if ctx else what
    if rc == -3:
        raise BudgetExceeded(rc, msg)
    raise McwError(rc, msg or what)
