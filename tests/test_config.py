"""config/main.conf parser: ConfigVal semantics (src/read/read_config.h:60-297)."""
import ctypes as C

from perigrain_gb300 import _native as N


def parse(text):
    c = N.Conf()
    N.lib().pg_conf_default(C.byref(c))
    rc = N.lib().pg_conf_read_string(C.byref(c), text.encode(), 1)
    return rc, c


def test_defaults():
    rc, c = parse("")
    assert rc == 0
    assert (c.timesteps, c.modulo, c.dt) == (8000, 100, 0.02 / 1e5)
    assert (c.is_parallel, c.do_resume, c.resume_ind, c.save_file, c.enable_fracture) == (1, 0, 50, 1, 0)
    assert (c.allow_damping, c.allow_friction, c.self_contact) == (1, 1, 1)
    assert (c.normal_stiffness, c.damping_ratio, c.friction_coefficient) == (-1, -1, -1)
    assert c.wall_top == -999 and c.wall_z_max == -999 and c.speed_wall_top == 0
    assert (c.set_movable_index, c.set_stoppable_index) == (-1, -1)


def test_whitespace_comments_and_values():
    rc, c = parse("# comment\n  timesteps = 2 50\n\nmodulo=10\n dt = 5e-8 \n#dt=1\nenable_fracture = 1\n"
                  "is_parallel = 0\nwall_top = 0.25\nspeed_wall_x_max=-1.5\nset_movable_index = 3\n"
                  "gradient_extforce = 7\nextforce_maxstep = 100\n")
    assert rc == 0
    assert c.timesteps == 250 and c.modulo == 10 and c.dt == 5e-8
    assert c.enable_fracture == 1 and c.is_parallel == 0
    assert c.wall_top == 0.25 and c.speed_wall_x_max == -1.5
    assert c.set_movable_index == 3 and c.gradient_extforce == 1 and c.extforce_maxstep == 100


def test_unknown_key_is_ignored_and_bad_value_fails():
    rc, c = parse("no_such_key = 3\ntimesteps = 12\n")
    assert rc == 0 and c.timesteps == 12
    rc, c = parse("timesteps = abc\n")
    assert rc == N.PG_EINVAL


def test_stoi_prefix_semantics():
    # std::stoi parses a leading integer; "1e-8" for an integer key gives 1
    rc, c = parse("modulo = 1e-8\nresume_ind = -1\n")
    assert rc == 0 and c.modulo == 1 and c.resume_ind == 2**32 - 1
