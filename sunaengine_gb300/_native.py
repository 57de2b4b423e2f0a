"""Build and load the CUDA engine library (libsuna_gb300.so) in-tree.

The library is compiled with nvcc for sm_103a only and loaded with ctypes.
There is no fallback: if the library cannot be built or loaded, every engine
call raises.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import threading
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / 'csrc'
BUILD = HERE / '_build'
LIB = BUILD / 'libsuna_gb300.so'
INCLUDE = HERE.parent / 'include'
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
_lock = threading.Lock()


def _sources():
    return sorted(CSRC.glob('*.cu')) + sorted(CSRC.glob('*.cuh')) + [INCLUDE / 'suna.h']


def nvcc() -> str:
    exe = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not Path(exe).exists():
        raise RuntimeError('nvcc not found: the CUDA engine cannot be built')
    return exe


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile csrc/*.cu into _build/libsuna_gb300.so (sm_103a): one nvcc per
    translation unit, run in parallel, then one link."""
    with _lock:
        srcs = _sources()
        if LIB.exists() and not force and all(LIB.stat().st_mtime >= s.stat().st_mtime for s in srcs):
            return LIB
        BUILD.mkdir(exist_ok=True)
        tag = os.getpid()
        # host floating point (the rigid-body record math restates JS doubles) without FMA contraction
        flags = [*ARCH, '-lineinfo', '-O3', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-ffp-contract=off',
                 '-diag-suppress', '550']
        if verbose:
            flags.append('-Xptxas=-v')
        units = sorted(CSRC.glob('*.cu'))
        objs = [BUILD / f'{u.stem}.{tag}.o' for u in units]
        procs = [subprocess.Popen([nvcc(), *flags, '-c', str(u), '-o', str(o)], stdout=subprocess.PIPE,
                                  stderr=subprocess.STDOUT, text=True) for u, o in zip(units, objs)]
        logs = [p.communicate()[0] for p in procs]
        bad = [(u, lg) for u, p, lg in zip(units, procs, logs) if p.returncode != 0]
        if verbose:
            for u, lg in zip(units, logs):
                print(f'--- {u.name}\n{lg}')
        if bad:
            for o in objs:
                o.unlink(missing_ok=True)
            raise RuntimeError('nvcc failed:\n' + '\n'.join(f'{u.name}:\n{lg}' for u, lg in bad))
        tmp = BUILD / f'libsuna_gb300.{tag}.so'
        r = subprocess.run([nvcc(), *ARCH, '-shared', '-o', str(tmp)] + [str(o) for o in objs],
                           capture_output=True, text=True)
        for o in objs:
            o.unlink(missing_ok=True)
        if r.returncode != 0:
            raise RuntimeError('nvcc link failed:\n' + r.stdout + r.stderr)
        os.replace(tmp, LIB)
        return LIB


class SnOpts(ctypes.Structure):
    _fields_ = [('max_particles', ctypes.c_uint32), ('max_cells', ctypes.c_uint32),
                ('iters', ctypes.c_uint32), ('debug', ctypes.c_uint32), ('chain', ctypes.c_uint32),
                ('device', ctypes.c_int32), ('luts', ctypes.c_void_p), ('mats', ctypes.c_void_p),
                ('mat_count', ctypes.c_uint32), ('lanes', ctypes.c_uint32)]


class SnScene(ctypes.Structure):
    _fields_ = [('n', ctypes.c_uint32), ('n_fluid', ctypes.c_uint32), ('pos', ctypes.c_void_p),
                ('vel', ctypes.c_void_p), ('mat_id', ctypes.c_void_p), ('flags', ctypes.c_void_p),
                ('temp', ctypes.c_void_p), ('fuel', ctypes.c_void_p), ('dom_w', ctypes.c_int32),
                ('dom_h', ctypes.c_int32), ('cell_shift', ctypes.c_uint32)]


class SnParticle(ctypes.Structure):
    _fields_ = [('x', ctypes.c_int32), ('y', ctypes.c_int32), ('vx', ctypes.c_int32), ('vy', ctypes.c_int32),
                ('mat', ctypes.c_int32), ('flags', ctypes.c_uint32), ('temp', ctypes.c_int32),
                ('fuel', ctypes.c_int32), ('has_temp', ctypes.c_uint32), ('has_fuel', ctypes.c_uint32)]


class SnInfo(ctypes.Structure):
    _fields_ = [('n', ctypes.c_uint32), ('n_fluid', ctypes.c_uint32), ('substep_count', ctypes.c_uint64),
                ('formation_clock', ctypes.c_uint64), ('grid_w', ctypes.c_uint32), ('grid_h', ctypes.c_uint32),
                ('cell_total', ctypes.c_uint32)]


# Every symbol include/suna.h declares, with its ctypes signature.
P = ctypes.c_void_p
u32, i32, u64, sz = ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_size_t
class Sn3Opts(ctypes.Structure):
    _fields_ = [('max_particles', ctypes.c_uint32), ('max_cells', ctypes.c_uint32),
                ('max_scenes', ctypes.c_uint32), ('iters', ctypes.c_uint32), ('debug', ctypes.c_uint32),
                ('chain', ctypes.c_uint32), ('device', ctypes.c_int32), ('luts', ctypes.c_void_p),
                ('mats', ctypes.c_void_p), ('mat_count', ctypes.c_uint32), ('lanes', ctypes.c_uint32)]


class Sn3Scene(ctypes.Structure):
    _fields_ = [('n', ctypes.c_uint32), ('pos', ctypes.c_void_p), ('vel', ctypes.c_void_p),
                ('mat', ctypes.c_void_p), ('gx', ctypes.c_uint32), ('gy', ctypes.c_uint32),
                ('gz', ctypes.c_uint32), ('stir_amp', ctypes.c_int32), ('frame', ctypes.c_uint32)]


class Sn3Info(ctypes.Structure):
    _fields_ = [('n', ctypes.c_uint32), ('cap', ctypes.c_uint32), ('gx', ctypes.c_uint32),
                ('gy', ctypes.c_uint32), ('gz', ctypes.c_uint32), ('iters', ctypes.c_uint32),
                ('substep_count', ctypes.c_uint64)]


SIGNATURES = {
    'sn_create': (ctypes.c_int, [ctypes.POINTER(SnOpts), ctypes.POINTER(P)]),
    'sn_destroy': (None, [P]),
    'sn_last_error': (ctypes.c_char_p, [P]),
    'sn_load_scene': (ctypes.c_int, [P, ctypes.POINTER(SnScene)]),
    'sn_step': (ctypes.c_int, [P, u32, ctypes.POINTER(u64)]),
    'sn_digest': (ctypes.c_int, [P, P]),
    'sn_chain': (ctypes.c_int, [P, P]),
    'sn_reset_chain': (ctypes.c_int, [P]),
    'sn_read_state': (ctypes.c_int, [P, P, sz]),
    'sn_read_scratch': (ctypes.c_int, [P, P, sz]),
    'sn_write_state': (ctypes.c_int, [P, P, P, sz]),
    'sn_read_bonds': (ctypes.c_int, [P, P, sz]),
    'sn_read_fields': (ctypes.c_int, [P, P, P, sz]),
    'sn_read_cell_start': (ctypes.c_int, [P, P, sz]),
    'sn_spawn': (ctypes.c_int, [P, P, u32, u32, ctypes.POINTER(u32)]),
    'sn_impulse': (ctypes.c_int, [P, i32, i32, i32, i32, i32, u32, ctypes.POINTER(u32)]),
    'sn_debug_counters': (ctypes.c_int, [P, P]),
    'sn_check_errors': (ctypes.c_int, [P]),
    'sn_sync': (ctypes.c_int, [P]),
    'sn_get_info': (ctypes.c_int, [P, ctypes.POINTER(SnInfo)]),
    'sn_set_formation_clock': (ctypes.c_int, [P, u64, u32]),
    'sn_set_walls': (ctypes.c_int, [P, u32, ctypes.POINTER(u32)]),
    'sn_last_timing': (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(u64)]),
    'sn_profile_substep': (ctypes.c_int, [P, u32, P, u32, ctypes.POINTER(u32)]),
    'sn_batch_profile_substep': (ctypes.c_int, [P, u32, P, u32, ctypes.POINTER(u32)]),
    'sn_batch_create': (ctypes.c_int, [ctypes.POINTER(SnOpts), u32, ctypes.POINTER(P)]),
    'sn_batch_destroy': (None, [P]),
    'sn_batch_last_error': (ctypes.c_char_p, [P]),
    'sn_batch_add_scene': (ctypes.c_int, [P, ctypes.POINTER(SnScene), u32, ctypes.POINTER(u32)]),
    'sn_batch_remove_scene': (ctypes.c_int, [P, u32]),
    'sn_batch_step': (ctypes.c_int, [P, u32]),
    'sn_batch_schedule_impulse': (ctypes.c_int, [P, u32, u64, i32, i32, i32, i32, i32, u32]),
    'sn_batch_digest': (ctypes.c_int, [P, u32, P]),
    'sn_batch_chain': (ctypes.c_int, [P, u32, P]),
    'sn_batch_read_state': (ctypes.c_int, [P, u32, P, sz]),
    'sn_batch_read_scratch': (ctypes.c_int, [P, u32, P, sz]),
    'sn_batch_write_state': (ctypes.c_int, [P, u32, P, P, sz, u64, u64, u32]),
    'sn_batch_get_info': (ctypes.c_int, [P, u32, ctypes.POINTER(SnInfo)]),
    'sn_batch_check_errors': (ctypes.c_int, [P]),
    'sn_batch_sync': (ctypes.c_int, [P]),
    'sn_batch_last_timing': (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(u64)]),
    'sn_digest_device_noalloc': (ctypes.c_int, [P, u32, u32, P, P, P]),
    'sn3_create': (ctypes.c_int, [ctypes.POINTER(Sn3Opts), ctypes.POINTER(P)]),
    'sn3_destroy': (None, [P]),
    'sn3_last_error': (ctypes.c_char_p, [P]),
    'sn3_load_scene': (ctypes.c_int, [P, ctypes.POINTER(Sn3Scene)]),
    'sn3_add_scene': (ctypes.c_int, [P, ctypes.POINTER(Sn3Scene), u32, ctypes.POINTER(u32)]),
    'sn3_remove_scene': (ctypes.c_int, [P, u32]),
    'sn3_step': (ctypes.c_int, [P, u32]),
    'sn3_spawn': (ctypes.c_int, [P, u32, P, P, u32, ctypes.POINTER(u32)]),
    'sn3_set_ball': (ctypes.c_int, [P, u32, u32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double]),
    'sn3_fnv': (ctypes.c_int, [P, u32, P]),
    'sn3_digest': (ctypes.c_int, [P, u32, P]),
    'sn3_chain': (ctypes.c_int, [P, u32, P]),
    'sn3_read_state': (ctypes.c_int, [P, u32, P, ctypes.c_size_t]),
    'sn3_write_bonds': (ctypes.c_int, [P, u32, P, ctypes.c_size_t, i32, i32]),
    'sn3_read_bonds': (ctypes.c_int, [P, u32, P, ctypes.c_size_t]),
    'sn3_write_state': (ctypes.c_int, [P, u32, P, u32, u64, P]),
    'sn3_debug_counters': (ctypes.c_int, [P, P]),
    'sn3_sync': (ctypes.c_int, [P]),
    'sn3_get_info': (ctypes.c_int, [P, u32, ctypes.POINTER(Sn3Info)]),
    'sn3_last_timing': (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(u64)]),
    'sn3_profile_substep': (ctypes.c_int, [P, u32, P, u32, ctypes.POINTER(u32)]),
    'sn_begin_weld_group': (ctypes.c_int, [P, ctypes.POINTER(u32)]),
    'sn_hold_weld_group': (ctypes.c_int, [P, u32]),
    'sn_end_weld_group': (ctypes.c_int, [P, ctypes.POINTER(u32)]),
    'sn_arm_fuse': (ctypes.c_int, [P, ctypes.POINTER(u32)]),
    'sn_weld_state': (ctypes.c_int, [P, P]),
    'sn_write_bonds': (ctypes.c_int, [P, P, ctypes.c_size_t]),
    'sn_batch_write_bonds': (ctypes.c_int, [P, u32, P, ctypes.c_size_t]),
    'sn_erase': (ctypes.c_int, [P, P, ctypes.c_size_t, ctypes.POINTER(u32)]),
    'sn_batch_erase': (ctypes.c_int, [P, u32, P, ctypes.c_size_t, ctypes.POINTER(u32)]),
    'sn_set_jets': (ctypes.c_int, [P, P, u32, ctypes.POINTER(u32)]),
    'sn_batch_set_jets': (ctypes.c_int, [P, u32, P, u32, ctypes.POINTER(u32)]),
    'sn_set_user_drive': (ctypes.c_int, [P, ctypes.c_int32, ctypes.c_int32, P]),
    'sn_make_rigid_body': (ctypes.c_int, [P, P, u32, P, u32, ctypes.POINTER(ctypes.c_int32)]),
    'sn_promote_weld_group': (ctypes.c_int, [P, u32, P, u32, ctypes.POINTER(ctypes.c_int32)]),
    'sn_end_weld_group_and_promote': (ctypes.c_int, [P, P, u32, ctypes.POINTER(ctypes.c_int32)]),
    'sn_dissolve_all_bodies': (ctypes.c_int, [P, ctypes.POINTER(u32)]),
    'sn_read_bodies': (ctypes.c_int, [P, P, ctypes.c_size_t, ctypes.POINTER(u32)]),
    'sn_read_rest_offsets': (ctypes.c_int, [P, P, ctypes.c_size_t]),
    'sn_set_body_user': (ctypes.c_int, [P, u32, u32, ctypes.POINTER(u32)]),
    'sn_set_body_driver': (ctypes.c_int, [P, u32, ctypes.c_int32, P]),
    'sn_clear_body_drivers': (ctypes.c_int, [P]),
    'sn_drag_body': (ctypes.c_int, [P, u32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.POINTER(u32)]),
    'sn_restore_bodies': (ctypes.c_int, [P, P, u32, P, ctypes.c_size_t]),
    'sn_batch_make_rigid_body': (ctypes.c_int, [P, u32, P, u32, P, u32, ctypes.POINTER(ctypes.c_int32)]),
    'sn_batch_promote_weld_group': (ctypes.c_int, [P, u32, u32, P, u32, ctypes.POINTER(ctypes.c_int32)]),
    'sn_batch_dissolve_all_bodies': (ctypes.c_int, [P, u32, ctypes.POINTER(u32)]),
    'sn_batch_read_bodies': (ctypes.c_int, [P, u32, P, ctypes.c_size_t, ctypes.POINTER(u32)]),
    'sn_batch_read_rest_offsets': (ctypes.c_int, [P, u32, P, ctypes.c_size_t]),
    'sn_batch_set_body_user': (ctypes.c_int, [P, u32, u32, u32, ctypes.POINTER(u32)]),
    'sn_batch_set_body_driver': (ctypes.c_int, [P, u32, u32, ctypes.c_int32, P]),
    'sn_batch_clear_body_drivers': (ctypes.c_int, [P, u32]),
    'sn_batch_drag_body': (ctypes.c_int, [P, u32, u32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                          ctypes.POINTER(u32)]),
    'sn_set_lanes': (ctypes.c_int, [P, P]),
    'sn_batch_set_lanes': (ctypes.c_int, [P, P]),
    'sn_set_material': (ctypes.c_int, [P, u32, P, ctypes.POINTER(u32)]),
    'sn_clear_materials': (ctypes.c_int, [P]),
    'sn_set_gravity_scale': (ctypes.c_int, [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
    'sn_batch_set_material': (ctypes.c_int, [P, u32, P, ctypes.POINTER(u32)]),
    'sn_write_body': (ctypes.c_int, [P, P, u32, u32, P, u32, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(u32)]),
    'sn_autotune': (ctypes.c_int, [P, u32, ctypes.POINTER(u32)]),
    'sn_batch_autotune': (ctypes.c_int, [P, u32, ctypes.POINTER(u32)]),
    'sn_set_staged': (ctypes.c_int, [P, u32]),
    'sn_set_tile_shape': (ctypes.c_int, [P, u32]),
    'sn_read_initial_positions': (ctypes.c_int, [P, P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    'sn_batch_set_tile_shape': (ctypes.c_int, [P, u32]),
    'sn_autotune_layout': (ctypes.c_int, [P, u32, ctypes.POINTER(u32), ctypes.POINTER(u32),
                                          ctypes.POINTER(ctypes.c_float)]),
    'sn_batch_autotune_layout': (ctypes.c_int, [P, u32, ctypes.POINTER(u32), ctypes.POINTER(u32),
                                                ctypes.POINTER(ctypes.c_float)]),
    'sn_batch_set_staged': (ctypes.c_int, [P, u32]),
    'sn_set_persistent': (ctypes.c_int, [P, u32]),
    'sn_batch_set_persistent': (ctypes.c_int, [P, u32]),
    'sn_lanes': (ctypes.c_int, [P, P]),
    'sn_batch_lanes': (ctypes.c_int, [P, P]),
    'sn_ckpt_pool_create': (ctypes.c_int, [ctypes.c_size_t, ctypes.c_int32, ctypes.POINTER(P)]),
    'sn_ckpt_pool_destroy': (None, [P]),
    'sn_ckpt_pool_last_error': (ctypes.c_char_p, [P]),
    'sn_ckpt_pool_usage': (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]),
    'sn_ckpt_free': (ctypes.c_int, [P, u64]),
    'sn_ckpt_bytes': (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_size_t)]),
    'sn_ckpt_save': (ctypes.c_int, [P, P, ctypes.POINTER(u64)]),
    'sn_ckpt_load': (ctypes.c_int, [P, P, u64]),
    'sn_batch_ckpt_bytes': (ctypes.c_int, [P, u32, ctypes.POINTER(ctypes.c_size_t)]),
    'sn_batch_ckpt_save': (ctypes.c_int, [P, u32, P, ctypes.POINTER(u64)]),
    'sn_batch_ckpt_load': (ctypes.c_int, [P, u32, P, u64]),
    'sn3_ckpt_bytes': (ctypes.c_int, [P, u32, ctypes.POINTER(ctypes.c_size_t)]),
    'sn3_ckpt_save': (ctypes.c_int, [P, u32, P, ctypes.POINTER(u64)]),
    'sn3_ckpt_load': (ctypes.c_int, [P, u32, P, u64]),
}

_lib = None


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libsuna_gb300.so (building it first if needed) and bind every symbol."""
    global _lib
    if _lib is None:
        path = build() if build_if_missing else LIB
        if not path.exists():
            raise RuntimeError(f'{path} is missing: run build() first')
        lib = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib
