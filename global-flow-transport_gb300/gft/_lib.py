"""ctypes binding of libgft.so (include/gft.h).

The library is the only compute path: importing this module fails loudly when
the shared object has not been built, and every call raises on a non-OK status.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libgft.so')

# gft_status -> exception, mirroring TF's InvalidArgument / Unimplemented / Internal
OK, ERR_INVALID_ARGUMENT, ERR_UNIMPLEMENTED, ERR_CUDA, ERR_WORKSPACE = 0, 1, 2, 3, 4


class GftError(RuntimeError):
    pass


class GftInvalidArgument(GftError, ValueError):
    pass


class GftUnimplemented(GftError, NotImplementedError):
    pass


class GftCudaError(GftError):
    pass


_EXC = {ERR_INVALID_ARGUMENT: GftInvalidArgument, ERR_UNIMPLEMENTED: GftUnimplemented,
        ERR_CUDA: GftCudaError, ERR_WORKSPACE: GftError}

_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_F = ctypes.c_float
_SZ = ctypes.c_size_t
_I64P = ctypes.POINTER(ctypes.c_int64)
_I32P = ctypes.POINTER(ctypes.c_int32)

# name -> (restype, argtypes)
_SIGS = {
    'gft_last_error': (ctypes.c_char_p, []),
    'gft_version': (ctypes.c_char_p, []),
    'gft_launch_count': (ctypes.c_ulonglong, []),
    'gft_set_knob': (_I32, [_I32, _I32]),
    'gft_get_knob': (_I32, [_I32]),
    'gft_raymarch_grid_transform': (_I32, [_P, _I32, _I64P, _P, _I32, _P, _P, _P, _I32, _I32P,
                                           _I32, _I32, _I32, _I32, _P, _P]),
    'gft_raymarch_grid_transform_store': (_I32, [_P, _I32, _I64P, _P, _I32, _P, _P, _P, _I32, _I32P,
                                                 _I32, _I32, _I32, _I32, _P, _P, _SZ, _P]),
    'gft_raymarch_grid_transform_samples_size': (_SZ, [_I64P, _I32, _I32P, _I32]),
    'gft_raymarch_grid_transform_samples_min_size': (_SZ, [_I64P, _I32, _I32P, _I32]),
    'gft_raymarch_grid_transform_grad_stored': (_I32, [_P, _I32, _I64P, _P, _P, _P, _I32, _P, _P, _P, _I32, _I32P,
                                                       _I32, _I32, _I32, _I32, _I32, _P, _SZ, _P, _P, _SZ, _P]),
    'gft_raymarch_grid_transform_grad_projected': (_I32, [_P, _I32, _I64P, _P, _P, _P, _I32, _P, _P, _P, _I32,
                                                          _I32P, _I32, _I32, _I32, _I32, _I32, _P, _SZ, _P, _P, _P,
                                                          _SZ, _P]),
    'gft_raymarch_grid_transform_grad_workspace_size': (_SZ, [_I64P, _I32, _I32, _I32]),
    'gft_raymarch_grid_transform_grad': (_I32, [_P, _I32, _I64P, _P, _P, _P, _I32, _P, _P, _P, _I32, _I32P,
                                                _I32, _I32, _I32, _I32, _I32, _P, _P, _SZ, _P]),
    'gft_raymarch_grid_transform_grad_weights': (_I32, [_I64P, _P, _I32, _P, _P, _P, _I32, _I32P, _I32, _I32,
                                                        _P, _SZ, _P]),
    'gft_raymarch_grid_transform_grad_weights_mode': (_I32, [_I64P, _P, _I32, _P, _P, _P, _I32, _I32P, _I32,
                                                             _I32, _I32, _P, _SZ, _P]),
    'gft_transmittance': (_I32, [_P, _I64P, _P, _P]),
    'gft_transmittance_grad': (_I32, [_P, _P, _I64P, _P, _P]),
    'gft_light_compose': (_I32, [_P, _P, _P, _I64P, _F, _F, _I32, _P, _P]),
    'gft_light_compose_grad': (_I32, [_P, _P, _P, _I64P, _F, _F, _I32, _P, _P, _P, _P]),
    'gft_light_compose_factored': (_I32, [_P, _P, _P, _P, _I64P, _F, _F, _I32, _P, _P]),
    'gft_light_compose_projection': (_I32, [_P, _F, _F, _P]),
    'gft_light_compose_factored_grad': (_I32, [_P, _P, _P, _I64P, _I32, _P, _P, _P, _P]),
    'gft_light_compose_factored_grad_cameras': (_I32, [_P, _P, _P, _I64P, _I32, _P, _P, _P, _P, _P]),
    'gft_image_loss_workspace_size': (_SZ, [ctypes.c_int64]),
    'gft_image_loss': (_I32, [_P, _P, _P, ctypes.c_int64, _P, _P, _SZ, _P]),
    'gft_image_loss_grad': (_I32, [_P, _P, _P, ctypes.c_int64, _P, _P, _P]),
    'gft_image_loss_tonemap': (_I32, [_P, _P, _P, ctypes.c_int64, _I32, _P, _P, _SZ, _P]),
    'gft_image_loss_tonemap_grad': (_I32, [_P, _P, _P, ctypes.c_int64, _I32, _P, _P, _P, _SZ, _P]),
    'gft_transmittance_check': (_I32, [_P, _P, _I64P, _I32, _P, _P]),
    'gft_raymarch_check': (_I32, [_P, _I32, _I64P, _P, _I32, _P, _P, _P, _I32, _I32P, _P, _I32, _P, _P]),
    'gft_raymarch_grid_transform_multi': (_I32, [_P, _I32, _I64P, _P, _I32, _P, _P, _P, _I32, _I32P,
                                                 _I32, _I32, _I32, _P, _P]),
    'gft_raymarch_grid_transform_multi_grad_workspace_size': (_SZ, [_I64P, _I32, _I32]),
    'gft_raymarch_grid_transform_multi_grad': (_I32, [_P, _I32, _I64P, _P, _P, _P, _I32, _P, _P, _P, _I32, _I32P,
                                                      _I32, _I32, _I32, _I32, _P, _P, _SZ, _P]),
    'gft_raymarch_grid_transform_multi_grad_weights': (_I32, [_I64P, _P, _I32, _P, _P, _P, _I32, _I32P, _I32, _P,
                                                              _SZ, _P]),
    'gft_raymarch_grid_transform_views': (_I32, [_P, _I32, _I64P, _P, _I32, _P, _P, _P, _I32, _I32P, _I32P,
                                                 _I32, _I32, _I32, _P, _P]),
    'gft_raymarch_grid_transform_views_grad_workspace_size': (_SZ, [_I64P, _I32, _I32]),
    'gft_raymarch_grid_transform_views_grad': (_I32, [_P, _I32, _I64P, _P, _P, _P, _I32, _P, _P, _P, _I32, _I32P,
                                                      _I32P, _I32, _I32, _I32, _I32, _P, _P, _SZ, _P]),
    'gft_raymarch_grid_transform_views_grad_weights': (_I32, [_I64P, _P, _I32, _P, _P, _P, _I32, _I32P, _I32P,
                                                              _I32, _P, _SZ, _P]),
    'gft_sample_grid_transform_workspace_size': (_SZ, [_I64P, _I32, _I32]),
    'gft_sample_grid_transform': (_I32, [_P, _I32, _I64P, _P, _I32, _P, _P, _P, _I32, _I32P,
                                         _I32, _I32, _I32, _I32, _F, _I32, _F, _I32, _P, _P, _SZ, _P]),
    'gft_sample_grid_transform_grad_workspace_size': (_SZ, [_I64P]),
    'gft_sample_grid_transform_grad': (_I32, [_I64P, _P, _I64P, _P, _I32, _P, _P, _P, _I32,
                                              _I32, _I32, _I32, _F, _I32, _I32, _P, _P, _SZ, _P]),
    'gft_sample_grid_lut_workspace_size': (_SZ, [_I64P, _I32, _I32]),
    'gft_sample_grid_lut': (_I32, [_P, _I32, _I64P, _P, _I64P, _I32, _I32, _I32, _I32, _F, _F,
                                   _I32, _I32, _I32, _P, _P, _SZ, _P]),
    'gft_sample_grid_lut_grad_workspace_size': (_SZ, [_I64P]),
    'gft_sample_grid_lut_grad': (_I32, [_P, _I64P, _P, _P, _I64P, _I32, _I32, _F, _I32, _I32, _I32, _I32,
                                        _P, _P, _P, _SZ, _P]),
    'gft_lod_transform': (_I32, [_I32P, _P, _P, _P, _I32, _I32P, _I32, _P, _P]),
    'gft_reduce_grid_blend': (_I32, [_P, _I64P, _I32, _I32, _P, _P]),
    'gft_reduce_grid_blend_grad': (_I32, [_P, _P, _P, _I64P, _I32, _I32, _I32, _P, _P]),
    'gft_advect_workspace_size': (_SZ, [_I64P, _I32]),
    'gft_advect': (_I32, [_P, _I32, _I64P, _P, _P, _P, _F, _I32, _I32, _I32, _P, _P, _SZ, _P]),
    'gft_advect_noalloc_max_elements': (_SZ, []),
    'gft_advect_noalloc': (_I32, [_P, _I32, _I64P, _P, _P, _P, _F, _I32, _I32, _I32, _P, _P]),
    'gft_advect_grad_workspace_size': (_SZ, [_I64P, _I32]),
    'gft_advect_grad_workspace_size_mode': (_SZ, [_I64P, _I32, _I32]),
    'gft_advect_grad': (_I32, [_P, _I64P, _P, _P, _P, _F, _I32, _I32, _I32, _I32, _P, _P, _P, _P, _P,
                               _P, _SZ, _P]),
}

_lib = None


def load(path=LIB_PATH):
    """Loads libgft.so once; raises ImportError when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError('libgft.so is not built (%s); run `python build.py` in the package directory '
                          'or __graft_entry__.build()' % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGS)


def check(status, what):
    if status != OK:
        msg = load().gft_last_error().decode(errors='replace')
        raise _EXC.get(status, GftError)('%s: %s' % (what, msg))


def i64(vals):
    vals = [int(v) for v in vals]
    return (ctypes.c_int64 * len(vals))(*vals)


def i32(vals):
    vals = [int(v) for v in vals]
    return (ctypes.c_int32 * len(vals))(*vals)
