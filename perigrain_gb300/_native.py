"""ctypes bindings of the C ABI (include/perigrain.h, include/perigrain_io.h).

The library is the in-tree ``libperigrain.so`` built by ``perigrain_gb300.build``. There is no
fallback: if the library is missing or cannot be loaded, every entry point raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libperigrain.so")

PG_OK, PG_EINVAL, PG_ENOMEM, PG_ECUDA, PG_ENAN, PG_ETIMEOUT, PG_EIO, PG_ECAPACITY, PG_ERANGE, PG_ENODEV = range(10)
PG_FP64, PG_MIXED = 0, 1
FIELD = {"CurrPos": 0, "vel": 1, "acc": 2, "force": 3, "disp": 4, "pos": 5}

u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)
u8p = C.POINTER(C.c_uint8)


class SetupDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_uint32), ("n_instances", C.c_uint32), ("n_grains", C.c_uint32), ("n_nodes", C.c_uint32),
        ("grain_instance", u32p), ("grain_node_offset", u32p),
        ("pos", f64p), ("vol", f64p), ("disp", f64p), ("vel", f64p), ("acc", f64p), ("extforce", f64p),
        ("bond_offset", u64p), ("bond_local", u32p),
        ("bdry_offset", u32p), ("bdry_nodes", u32p), ("clamped_offset", u32p), ("clamped_nodes", u32p),
        ("delta", f64p), ("rho", f64p), ("cnot", f64p), ("snot", f64p),
        ("movable", i32p), ("breakable", i32p), ("stoppable", i32p), ("break_bonds", u8p),
        ("torque_axis", u32p), ("torque_val", f64p),
        ("contact_radius", f64p), ("normal_stiffness", f64p), ("friction_coefficient", f64p),
        ("damping_ratio", f64p),
        ("allow_wall", i32p), ("wall_geom", f64p), ("wall_speed", f64p),
    ]


class Config(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("enable_fracture", C.c_int32), ("nl_bdry_only", C.c_int32),
        ("allow_damping", C.c_int32), ("allow_friction", C.c_int32), ("self_contact", C.c_int32),
        ("enable_torque", C.c_int32), ("gradient_extforce", C.c_int32), ("extforce_maxstep", C.c_uint32),
        ("precision", C.c_int32), ("record_pairs", C.c_int32), ("pair_log_capacity", C.c_uint32),
        ("first_step", C.c_uint32), ("max_contacts", C.c_uint32), ("block_size", C.c_uint32),
        ("autotune", C.c_int32), ("cells_per_node", C.c_uint32), ("contact_skin", C.c_double),
        ("timeloop", C.c_int32), ("node_order", C.c_int32),
    ]


NODE_ORDER = {"input": 0, "cell": 1, "cell_degree": 2, "shuffle": 3, "cell_block_degree": 4}

CONF_FIELDS = [
    ("timesteps", C.c_uint32), ("modulo", C.c_uint32), ("dt", C.c_double),
    ("is_parallel", C.c_int32), ("do_resume", C.c_int32), ("wall_resume", C.c_int32),
    ("resume_ind", C.c_uint32), ("save_file", C.c_int32), ("enable_fracture", C.c_int32),
    ("nl_bdry_only", C.c_int32), ("allow_damping", C.c_int32), ("allow_friction", C.c_int32),
    ("normal_stiffness", C.c_double), ("damping_ratio", C.c_double), ("friction_coefficient", C.c_double),
    ("self_contact", C.c_int32), ("self_contact_rad", C.c_double), ("enable_torque", C.c_int32),
    ("set_movable_index", C.c_int32), ("set_movable_timestep", C.c_int32),
    ("set_stoppable_index", C.c_int32), ("set_stoppable_timestep", C.c_int32),
    ("reset_partzero_y", C.c_int32), ("reset_partzero_y_timestep", C.c_uint32), ("wheel_rad", C.c_double),
    ("wall_left", C.c_double), ("wall_right", C.c_double), ("wall_top", C.c_double), ("wall_bottom", C.c_double),
    ("wall_x_min", C.c_double), ("wall_y_min", C.c_double), ("wall_z_min", C.c_double),
    ("wall_x_max", C.c_double), ("wall_y_max", C.c_double), ("wall_z_max", C.c_double),
    ("speed_wall_left", C.c_double), ("speed_wall_right", C.c_double), ("speed_wall_top", C.c_double),
    ("speed_wall_bottom", C.c_double),
    ("speed_wall_x_min", C.c_double), ("speed_wall_y_min", C.c_double), ("speed_wall_z_min", C.c_double),
    ("speed_wall_x_max", C.c_double), ("speed_wall_y_max", C.c_double), ("speed_wall_z_max", C.c_double),
    ("gradient_extforce", C.c_int32), ("extforce_maxstep", C.c_uint32),
]


class PackMesh(C.Structure):
    _fields_ = [("dim", C.c_uint32), ("n_nodes", C.c_uint32), ("n_elems", C.c_uint32), ("pos", C.c_void_p),
                ("elems", C.c_void_p), ("n_bdry_nodes", C.c_uint32), ("bdry_nodes", C.c_void_p),
                ("n_bdry_edges", C.c_uint32), ("bdry_edges", C.c_void_p)]


class Post(C.Structure):
    _fields_ = [(k, f64p) for k in ("grain_mean_vel", "grain_mean_acc", "grain_mean_currpos", "grain_force",
                                    "grain_damage", "node_damage", "inertial_force", "volume_fraction")]


class Conf(C.Structure):
    _fields_ = CONF_FIELDS


class SnapshotDesc(C.Structure):
    _fields_ = [("currpos", C.c_void_p), ("vel", C.c_void_p), ("acc", C.c_void_p), ("force", C.c_void_p),
                ("disp", C.c_void_p), ("bond_alive", C.c_void_p), ("wall", C.c_void_p), ("reaction", C.c_void_p),
                ("too_close_events", C.c_void_p), ("last_step", C.c_void_p)]


# (name, restype, argtypes) of every exported function; tests check that each is exported.
PROTOTYPES = [
    ("pg_version", C.c_int, []),
    ("pg_device_count", C.c_int, [i32p]),
    ("pg_status_string", C.c_char_p, [C.c_int]),
    ("pg_last_error", C.c_char_p, []),
    ("pg_config_default", None, [C.POINTER(Config)]),
    ("pg_select_device", C.c_int, [C.c_int]),
    ("pg_create", C.c_int, [C.POINTER(SetupDesc), C.POINTER(Config), C.POINTER(C.c_void_p)]),
    ("pg_destroy", C.c_int, [C.c_void_p]),
    ("pg_step", C.c_int, [C.c_void_p, C.c_uint32]),
    ("pg_synchronize", C.c_int, [C.c_void_p]),
    ("pg_step_timed", C.c_int, [C.c_void_p, C.c_uint32, f64p]),
    ("pg_get_step", C.c_int, [C.c_void_p, u64p]),
    ("pg_get_field", C.c_int, [C.c_void_p, C.c_int, f64p]),
    ("pg_set_field", C.c_int, [C.c_void_p, C.c_int, f64p]),
    ("pg_get_bond_alive", C.c_int, [C.c_void_p, u8p]),
    ("pg_get_bond_break_step", C.c_int, [C.c_void_p, u32p]),
    ("pg_set_bond_alive", C.c_int, [C.c_void_p, u8p]),
    ("pg_get_reaction", C.c_int, [C.c_void_p, f64p]),
    ("pg_get_wall", C.c_int, [C.c_void_p, f64p]),
    ("pg_set_wall", C.c_int, [C.c_void_p, f64p]),
    ("pg_set_grain_flags", C.c_int, [C.c_void_p, C.c_uint32, C.c_int32, C.c_int32]),
    ("pg_snapshot", C.c_int, [C.c_void_p, C.POINTER(SnapshotDesc)]),
    ("pg_wait", C.c_int, [C.c_void_p]),
    ("pg_host_alloc", C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    ("pg_host_free", C.c_int, [C.c_void_p]),
    ("pg_get_pair_log", C.c_int, [C.c_void_p, C.c_uint32, u64p, u64p]),
    ("pg_get_device_status", C.c_int, [C.c_void_p, i32p, u64p]),
    ("pg_debug_grid_barrier", C.c_int, [C.c_void_p, C.c_uint32]),
    ("pg_debug_ieee64", C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    ("pg_get_launch_count", C.c_int, [C.c_void_p, u64p]),
    ("pg_get_launch_config", C.c_int, [C.c_void_p, u32p, u32p]),
    ("pg_get_contact_skin", C.c_int, [C.c_void_p, f64p]),
    ("pg_get_node_order", C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    ("pg_debug_node_order", C.c_int, [C.POINTER(SetupDesc), C.c_int32, C.c_void_p, C.POINTER(C.c_int32)]),
    ("pg_set_timing", C.c_int, [C.c_void_p, C.c_int32]),
    ("pg_get_kernel_times", C.c_int, [C.c_void_p, f64p, f64p, u64p]),
    ("pg_build_bonds", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_void_p, C.c_uint64, u64p,
                                 C.c_void_p]),
    ("pg_bond_last_error", C.c_char_p, []),
    ("pg_build_bonds_noalloc", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_double, C.c_void_p, C.c_uint64,
                                         u64p, C.c_void_p]),
    ("pg_noalloc_last_error", C.c_char_p, []),
    ("pg_postprocess", C.c_int, [C.c_void_p, C.c_void_p]),
    ("pg_pack_incenters", C.c_int, [C.POINTER(PackMesh), C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, u32p, u32p,
                                    C.c_void_p]),
    ("pg_pack_last_error", C.c_char_p, []),
    # gradients
    ("pg_set_grain_params", C.c_int, [C.c_void_p, f64p, f64p, f64p, f64p, f64p]),
    ("pg_get_grain_params", C.c_int, [C.c_void_p, f64p, f64p, f64p, f64p, f64p]),
    ("pg_grad_begin", C.c_int, [C.c_void_p]),
    ("pg_grad_reset", C.c_int, [C.c_void_p]),
    ("pg_masks_record", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_void_p)]),
    ("pg_masks_free", None, [C.c_void_p]),
    ("pg_grad_forward", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]),
    ("pg_grad_backward", C.c_int, [C.c_void_p, f64p, f64p, f64p, f64p]),
    ("pg_grad_times", C.c_int, [C.c_void_p, f64p, f64p, u64p, u64p]),
    # perigrain_io.h
    ("pg_conf_default", None, [C.POINTER(Conf)]),
    ("pg_conf_read_file", C.c_int, [C.POINTER(Conf), C.c_char_p]),
    ("pg_conf_read_string", C.c_int, [C.POINTER(Conf), C.c_char_p, C.c_int]),
    ("pg_setup_load", C.c_int, [C.c_char_p, C.c_uint32, C.c_int32, C.POINTER(C.c_void_p)]),
    ("pg_setup_from_desc", C.c_int, [C.POINTER(SetupDesc), C.POINTER(C.c_void_p)]),
    ("pg_setup_free", C.c_int, [C.c_void_p]),
    ("pg_setup_desc_get", C.c_int, [C.c_void_p, C.POINTER(SetupDesc)]),
    ("pg_setup_apply_conf", C.c_int, [C.c_void_p, C.POINTER(Conf)]),
    ("pg_setup_save", C.c_int, [C.c_void_p, C.c_char_p]),
    ("pg_setup_set_connectivity", C.c_int, [C.c_void_p, C.c_uint32, u32p, C.c_uint64]),
    ("pg_write_snapshot", C.c_int, [C.c_void_p, C.c_void_p, C.c_char_p, C.c_uint32]),
    ("pg_write_tc", C.c_int, [C.c_void_p, C.c_char_p, C.c_uint32, f64p, f64p, f64p, f64p, u8p, f64p, f64p,
                              C.c_int32]),
    ("pg_run_simulation", C.c_int, [C.c_char_p, C.c_uint32, C.c_int32]),
    ("pg_h5w_new", C.c_void_p, []),
    ("pg_h5w_add", C.c_int, [C.c_void_p, C.c_char_p, C.c_int32, C.c_uint32, u64p, C.c_void_p]),
    ("pg_h5w_group", C.c_int, [C.c_void_p, C.c_char_p]),
    ("pg_h5w_write", C.c_int, [C.c_void_p, C.c_char_p]),
    ("pg_h5w_free", None, [C.c_void_p]),
    ("pg_h5_info", C.c_int, [C.c_char_p, C.c_char_p, u32p, u64p, i32p, u32p, i32p]),
    ("pg_h5_read", C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.c_void_p, C.c_uint64]),
    ("pg_h5_list", C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_uint64]),
]

_lib = None


class PerigrainError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("perigrain status %d: %s" % (code, msg))
        self.code = code


def lib():
    """Load libperigrain.so (raises if it is missing -- there is no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("perigrain_gb300 native library not built: %s (run perigrain_gb300.build.build())"
                              % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, res, args in PROTOTYPES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != PG_OK:
        msg = lib().pg_last_error()
        raise PerigrainError(rc, msg.decode() if msg else "")
    return rc


def ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))
