"""Build and bind the C-ABI library ``libdmgb300.so`` (declared in include/dm_gb300.h).

The library is compiled in-tree for sm_103a only (``build()``), with the
translation units compiled in parallel and linked with ``nvcc -shared``.
``lib()`` loads it with ctypes; the signatures below mirror the header.
There is no fallback: if the library is missing or fails to load, every
entry point of the package raises.
"""
import ctypes
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, 'csrc')
INCLUDE = os.path.join(REPO_DIR, 'include')
BUILD_DIR = os.path.join(PKG_DIR, '_build')
LIB_PATH = os.path.join(PKG_DIR, 'libdmgb300.so')
SOURCES = ['dm_misc.cu', 'dm_pass.cu', 'dm_state.cu', 'dm_measure.cu', 'dm_tc.cu', 'dm_tma.cu', 'dm_mlp.cu',
           'dm_sample.cu', 'dm_sched.cpp']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', '-Xptxas', '-warn-spills',
              '--expt-relaxed-constexpr']

DM_OK, DM_ERR_ARG, DM_ERR_CUDA, DM_ERR_RANGE, DM_ERR_PROGRAM = 0, -1, -2, -3, -4
DM_F64, DM_F32 = 0, 1
DM_MAX_QUBITS = 17
DM_MAX_TILE_AXES = 7
DM_MAX_PASS_OPS = 128
DM_MAX_ROUNDS = 48
DM_ROUND_AXES = {0: 2, 1: 3}     # dtype -> axes per register round
DM_OP_MAP1, DM_OP_MAP2, DM_OP_DIAG2, DM_OP_CX = 1, 2, 3, 4
DM_MAP1_ROW0_IDENTITY = 1
DM_MAP1_XY_UNITAL = 2
DM_CX_IDEAL = 1
DM_IMAGE_TC, DM_IMAGE_TMA = 1, 2
DM_SCHED_GATE1, DM_SCHED_CX, DM_SCHED_MEASURE, DM_SCHED_RESET, DM_SCHED_BARRIER, DM_SCHED_OTHER = 1, 2, 3, 4, 5, 6


class NativeError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, fn, code, msg):
        super().__init__('%s failed: %s (%d)' % (fn, msg, code))
        self.code = code


def _nvcc():
    for cand in (os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc'):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return 'nvcc'


def build(force=False, verbose=False):
    """Compile csrc/*.cu for sm_103a and link libdmgb300.so in the package directory."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cuh')] \
        + [os.path.join(INCLUDE, 'dm_gb300.h')]
    newest = max(os.path.getmtime(d) for d in deps)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + '.o')
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ['-I', INCLUDE, '-I', CSRC, '-c', src, '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, ' '.join(cmd), r.stderr))
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + '.tmp'
    cmd = [nvcc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lcudart_static', '-lrt', '-ldl', '-lpthread']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc link failed:\n%s\n%s' % (' '.join(cmd), r.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class DmOp(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int32), ('a', ctypes.c_int16), ('b', ctypes.c_int16),
                ('flags', ctypes.c_int32), ('moff', ctypes.c_int32)]


class DmPass(ctypes.Structure):
    _fields_ = [('k', ctypes.c_int32), ('axes', ctypes.c_int32 * DM_MAX_TILE_AXES),
                ('nops', ctypes.c_int32), ('nrounds', ctypes.c_int32),
                ('round_axes', (ctypes.c_int8 * 4) * DM_MAX_ROUNDS),
                ('round_end', ctypes.c_int16 * DM_MAX_ROUNDS),
                ('ops', DmOp * DM_MAX_PASS_OPS)]


class DmTcRound(ctypes.Structure):
    _fields_ = [('digits', ctypes.c_int8 * 3), ('vec', ctypes.c_int8), ('umoff', ctypes.c_int32),
                ('rowc', ctypes.c_uint32 * 8), ('kc', ctypes.c_uint32 * 6)]


class DmTcPass(ctypes.Structure):
    _fields_ = [('axes', ctypes.c_int32 * 7), ('nrounds', ctypes.c_int32), ('vec0', ctypes.c_int8),
                ('direct_last', ctypes.c_int8), ('pad', ctypes.c_int8 * 2), ('natrow', ctypes.c_uint32 * 8), ('natk', ctypes.c_uint32 * 6),
                ('rounds', DmTcRound * DM_MAX_ROUNDS)]


class DmBatchPass(ctypes.Structure):
    _fields_ = [('k', ctypes.c_int8), ('nrounds', ctypes.c_int8), ('nops', ctypes.c_int16),
                ('axes', ctypes.c_int8 * DM_MAX_TILE_AXES), ('pad', ctypes.c_int8),
                ('round_axes', (ctypes.c_int8 * 4) * DM_MAX_ROUNDS),
                ('round_end', ctypes.c_int16 * DM_MAX_ROUNDS),
                ('ops', DmOp * DM_MAX_PASS_OPS)]


class DmBatchTcPass(ctypes.Structure):
    _fields_ = [('ops', DmBatchPass), ('tables', DmTcPass)]


class DmBatchInstance(ctypes.Structure):
    _fields_ = [('n', ctypes.c_int32), ('npasses', ctypes.c_int32), ('pass_begin', ctypes.c_int32),
                ('pad', ctypes.c_int32), ('state_off', ctypes.c_int64), ('prob_off', ctypes.c_int64),
                ('mats_off', ctypes.c_int64), ('mats_len', ctypes.c_int64), ('meas_err', ctypes.c_double)]


class DmRecipe(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int8), ('nrot', ctypes.c_int8), ('axis', ctypes.c_int8 * 3),
                ('pad', ctypes.c_int8 * 3), ('const_off', ctypes.c_int32), ('pad2', ctypes.c_int32),
                ('angle', ctypes.c_double * 3)]


class DmParamSlot(ctypes.Structure):
    _fields_ = [('begin', ctypes.c_int32), ('len', ctypes.c_int32)]


class DmParamProgram(ctypes.Structure):
    _fields_ = [('n', ctypes.c_int32), ('npasses', ctypes.c_int32), ('nslots', ctypes.c_int32),
                ('nchain', ctypes.c_int32), ('nrecipes', ctypes.c_int32), ('nconsts', ctypes.c_int32),
                ('passes', ctypes.c_void_p), ('slots', ctypes.c_void_p), ('chain', ctypes.c_void_p),
                ('recipes', ctypes.c_void_p), ('consts', ctypes.c_void_p)]


DM_PARAMS_MIN_STRIDE = 12
DM_RECIPE_ROT, DM_RECIPE_NOISE, DM_RECIPE_CX, DM_RECIPE_CONST = 1, 2, 3, 4


class DmMlpGemm(ctypes.Structure):
    _fields_ = [('epi', ctypes.c_int32), ('M', ctypes.c_int32), ('N', ctypes.c_int32), ('K', ctypes.c_int32),
                ('members', ctypes.c_int32), ('pad', ctypes.c_int32),
                ('A', ctypes.c_void_p), ('lda', ctypes.c_int64), ('a_ms', ctypes.c_int64),
                ('B', ctypes.c_void_p), ('ldb', ctypes.c_int64), ('b_ms', ctypes.c_int64),
                ('bias', ctypes.c_void_p), ('bias_ms', ctypes.c_int64),
                ('pre', ctypes.c_void_p), ('ld_pre', ctypes.c_int64), ('pre_ms', ctypes.c_int64),
                ('out_f32', ctypes.c_void_p), ('ld_f32', ctypes.c_int64), ('f32_ms', ctypes.c_int64),
                ('out_bf16', ctypes.c_void_p), ('ld_bf16', ctypes.c_int64), ('bf16_ms', ctypes.c_int64),
                ('out_t', ctypes.c_void_p), ('ld_t', ctypes.c_int64), ('t_ms', ctypes.c_int64)]


DM_MLP_EPI_GELU_FWD, DM_MLP_EPI_BIAS_F32, DM_MLP_EPI_GELU_BWD, DM_MLP_EPI_F32 = 0, 1, 2, 3

_vp = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double
_sz = ctypes.c_size_t
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_i64p = ctypes.POINTER(ctypes.c_int64)

SIGNATURES = {
    'dm_init_product': (_i, [_vp, _i, _i, _dp, _d, _vp]),
    'dm_load_state': (_i, [_vp, _i, _i, _dp, _vp]),
    'dm_apply_map1': (_i, [_vp, _i, _i, _i, _dp, _vp]),
    'dm_apply_cx': (_i, [_vp, _i, _i, _i, _i, _dp, _vp]),
    'dm_apply_memory_noise': (_i, [_vp, _i, _i, _d, _d, _d, _vp]),
    'dm_apply_pass': (_i, [_vp, _i, _i, ctypes.POINTER(DmPass), _vp, _sz, _vp]),
    'dm_apply_pass_tc': (_i, [_vp, _i, ctypes.POINTER(DmTcPass), _vp, _sz, _vp, _vp]),
    'dm_apply_pass_tma': (_i, [_vp, _i, ctypes.POINTER(DmTcPass), _vp, _sz, _vp, _vp]),
    'dm_compose_rounds': (_i, [_i, ctypes.POINTER(DmBatchPass), _vp, _sz, _vp, _sz, _vp]),
    'dm_max_abs_diff': (_i, [_vp, _i, _vp, _i, _i, _vp, _vp]),
    'dm_tile_copy_probe': (_i, [_vp, _i, _vp, _vp]),
    'dm_fp64_fma_probe_threads': (_i, []),
    'dm_fp64_fma_probe': (_i, [_vp, ctypes.c_int64, _vp]),
    'dm_levelize': (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    'dm_host_alloc': (_vp, [_sz]),
    'dm_host_device_pointer': (_vp, [_vp]),
    'dm_host_free': (_i, [_vp]),
    'dm_tc_wait_selftest': (_i, [_vp, ctypes.c_int64, _vp]),
    'dm_batch_run': (_i, [_i, _vp, _sz, _vp, _sz, _vp, _sz, ctypes.POINTER(DmBatchInstance), _vp, _i,
                          ctypes.POINTER(DmBatchPass), _vp, _i, _vp, _vp, _vp]),
    'dm_batch_tc_scratch_bytes': (_sz, []),
    'dm_batch_run_tc': (_i, [_vp, _sz, _vp, _sz, _vp, _sz, ctypes.POINTER(DmBatchInstance), _vp, _i,
                             ctypes.POINTER(DmBatchTcPass), _vp, _i, _vp, _vp, _sz, _vp, _vp]),
    'dm_batch_run_params_tc': (_i, [ctypes.POINTER(DmParamProgram), ctypes.POINTER(DmParamProgram),
                                    ctypes.POINTER(DmBatchTcPass), _vp, _vp, _i, _i, _vp, _sz, _vp, _sz, _vp, _vp,
                                    _sz, _vp, _vp]),
    'dm_batch_run_params': (_i, [_i, ctypes.POINTER(DmParamProgram), ctypes.POINTER(DmParamProgram), _vp, _i, _i,
                                 _vp, _sz, _vp, _sz, _vp, _vp]),
    'dm_mlp_gemm_run': (_i, [ctypes.POINTER(DmMlpGemm), _vp, _vp]),
    'dm_mlp_softmax_xent': (_i, [_vp, _vp, _i, _i, _i, ctypes.c_float, _vp, _vp, _vp, _vp, _vp]),
    'dm_mlp_bias_grad': (_i, [_vp, ctypes.c_int64, ctypes.c_int64, _i, _i, _i, _vp, ctypes.c_int64, _vp]),
    'dm_mlp_adam': (_i, [_vp, _vp, _vp, _vp, ctypes.c_int64, _i, ctypes.POINTER(ctypes.c_int32), _i, ctypes.c_float,
                         ctypes.c_float, ctypes.c_float, ctypes.c_float, _i, _vp, _vp, _vp]),
    'dm_mlp_gather': (_i, [_vp, _i, _vp, _i, ctypes.c_int64, _vp, _i, _i, _i, _vp, _vp, _vp, _vp]),
    'dm_mlp_ensemble': (_i, [_vp, _i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    'dm_axis_probs': (_i, [_vp, _i, _i, _ip, _d, _vp, _vp]),
    'dm_nbasis_probs_scratch_bytes': (_sz, [_i]),
    'dm_nbasis_probs': (_i, [_vp, _i, _i, _dp, _d, _vp, _vp, _vp]),
    'dm_nbasis_probs_noalloc': (_i, [_vp, _i, _i, _dp, _d, _vp, _vp]),
    'dm_gather': (_i, [_vp, _i, _i, _i64p, _i, _vp, _vp]),
    'dm_sample_counts_scratch_bytes': (_sz, [_i]),
    'dm_sample_counts': (_i, [_vp, _i, ctypes.c_int64, ctypes.c_uint64, _vp, _vp, _vp]),
    'dm_chop_copy': (_i, [_vp, _i, _i, _d, _vp, _vp]),
    'dm_chop_copy_range': (_i, [_vp, _i, _i, ctypes.c_int64, ctypes.c_int64, _d, _vp, _vp]),
    'dm_pauli_to_matrix_scratch_bytes': (_sz, [_i]),
    'dm_pauli_to_matrix': (_i, [_vp, _i, _i, _vp, _vp, _vp]),
    'dm_overlap_scratch_bytes': (_sz, [_i]),
    'dm_overlap': (_i, [_vp, _vp, _i, _i, _vp, _vp, _vp]),
    'dm_error_string': (ctypes.c_char_p, [_i]),
    'dm_kernel_launch_count': (ctypes.c_uint64, []),
    'dm_version': (ctypes.c_char_p, []),
}

_LIB = None


def lib():
    """Load libdmgb300.so (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise NativeError('load', DM_ERR_ARG, 'libdmgb300.so is not built (run build())')
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def call(name, *args):
    """Call an int-returning entry point and raise NativeError on a non-zero status."""
    L = lib()
    rc = getattr(L, name)(*args)
    if rc != DM_OK:
        raise NativeError(name, rc, L.dm_error_string(rc).decode())
    return rc


def f64_array(values):
    arr = (ctypes.c_double * len(values))(*[float(v) for v in values])
    return arr
