/*
 * perigrain_io.h -- the process/file contract of the reference simulator, as a C ABI.
 *
 *   config/main.conf   key = value parser          (reference src/read/read_config.h:14-297)
 *   data/hdf5/all.h5   setup loader                (src/read/load_hdf5.h:28-201)
 *   output/hdf5/       plotinfo / tc_ / wall_ / run_time writers (src/particle/timeloop.h:560-582,
 *                      :881-1014)
 *   run_timeloop       the whole driver on top of perigrain.h (src/particle/timeloop.h:501-1015,
 *                      run/simulate2d.cpp:31-94)
 *
 * HDF5 is read and written by the project's own HDF5-subset library (h5lite); the files are
 * standard HDF5 (superblock v0, symbol-table groups, contiguous datasets).
 */
#ifndef PERIGRAIN_IO_H
#define PERIGRAIN_IO_H

#include <stddef.h>
#include <stdint.h>

#include "perigrain.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ConfigVal (read_config.h:14-119): every key of the reference, same defaults, same sentinels
 * (-1 for contact overrides, -999 for wall overrides). Booleans are 0/1. */
typedef struct pg_conf {
  uint32_t timesteps, modulo;
  double dt;
  int32_t is_parallel, do_resume, wall_resume;
  uint32_t resume_ind;
  int32_t save_file, enable_fracture, nl_bdry_only;
  int32_t allow_damping, allow_friction;
  double normal_stiffness, damping_ratio, friction_coefficient;
  int32_t self_contact;
  double self_contact_rad;
  int32_t enable_torque;
  int32_t set_movable_index, set_movable_timestep, set_stoppable_index, set_stoppable_timestep;
  int32_t reset_partzero_y;
  uint32_t reset_partzero_y_timestep;
  double wheel_rad;
  double wall_left, wall_right, wall_top, wall_bottom;
  double wall_x_min, wall_y_min, wall_z_min, wall_x_max, wall_y_max, wall_z_max;
  double speed_wall_left, speed_wall_right, speed_wall_top, speed_wall_bottom;
  double speed_wall_x_min, speed_wall_y_min, speed_wall_z_min;
  double speed_wall_x_max, speed_wall_y_max, speed_wall_z_max;
  int32_t gradient_extforce;
  uint32_t extforce_maxstep;
} pg_conf;

void pg_conf_default(pg_conf* c);
/* ConfigVal::read_file (read_config.h:122-297): whitespace removed, '#' comments, unknown key
 * -> "Error: Wrong config name: <k> !!" on stderr; missing file -> message on stderr, defaults
 * kept (returns PG_OK); a value that does not parse returns PG_EINVAL. */
int pg_conf_read_file(pg_conf* c, const char* path);
/* Parse from a string (same rules); `quiet` suppresses the stdout/stderr messages. */
int pg_conf_read_string(pg_conf* c, const char* text, int quiet);

/* ---- setup (all.h5) ---------------------------------------------------------------------- */
typedef struct pg_setup pg_setup;
/* load_particles/load_contact/load_wall for one simulation (dim 2 or 3). Grains are read from
 * groups P_00001.. (1-based). break_bonds is set to 1 for every grain, as run/simulate2d.cpp
 * does (the project's 3D driver does the same). */
int pg_setup_load(const char* all_h5, uint32_t dim, int32_t load_torque, pg_setup** out);
/* Build a setup from arrays (same layout as pg_setup_desc, one instance); copies everything. */
int pg_setup_from_desc(const pg_setup_desc* d, pg_setup** out);
int pg_setup_free(pg_setup* s);
/* Borrow a descriptor whose pointers stay valid until the setup is freed or modified. */
int pg_setup_desc_get(pg_setup* s, pg_setup_desc* d);
/* Contact.apply_config / RectWall.apply_config (contact.h:85-108, :254-301). */
int pg_setup_apply_conf(pg_setup* s, const pg_conf* c);
/* Write the setup as all.h5 in the layout of Experiment.save (exp_dict.py:705-768). */
int pg_setup_save(pg_setup* s, const char* all_h5);
/* Replace grain g's bond rows by conn2NArr(conn) (load_hdf5.h:28-38); conn is m x 2 local ids. */
int pg_setup_set_connectivity(pg_setup* s, uint32_t grain, const uint32_t* conn, uint64_t m);

/* ---- output ------------------------------------------------------------------------------ */
/* Write tc_%05u.h5 + wall_%05u.h5 for `counter` into out_dir from a live handle. */
int pg_write_snapshot(pg_handle* h, pg_setup* s, const char* out_dir, uint32_t counter);
/* The same files from host arrays laid out as pg_snapshot_desc fills them: n_nodes*dim fields,
 * bond_alive in CSR order (null: every bond of the setup is intact), wall [2*dim], reaction
 * [2*dim*dim]. connectivity = 0 leaves Connectivity out, as run_timeloop_worm does. */
int pg_write_tc(pg_setup* s, const char* out_dir, uint32_t counter, const double* currpos, const double* vel,
                const double* acc, const double* force, const uint8_t* bond_alive, const double* wall,
                const double* reaction, int32_t connectivity);

/* ---- the driver -------------------------------------------------------------------------- */
/* run/simulate{2,3}d: read <root>/config/main.conf and <root>/data/hdf5/all.h5, run the time
 * loop on the GPU and write <root>/output/hdf5/. Prints the reference's messages, progress
 * table and "Runtime: Ns". precision: pg_precision. Returns a pg_status. */
int pg_run_simulation(const char* root, uint32_t dim, int32_t precision);

/* ---- HDF5 subset (for tools and tests) ---------------------------------------------------- */
typedef struct pg_h5w pg_h5w;
/* dtype codes: 0 f64, 1 f32, 2 u32, 3 i32, 4 u64, 5 i64, 6 u8 */
pg_h5w* pg_h5w_new(void);
int pg_h5w_add(pg_h5w* w, const char* path, int32_t dtype, uint32_t rank, const uint64_t* dims,
               const void* data);
int pg_h5w_group(pg_h5w* w, const char* path);
int pg_h5w_write(pg_h5w* w, const char* filename);
void pg_h5w_free(pg_h5w* w);
/* Dataset shape and stored type: class 0 fixed point / 1 float, element size, signedness. */
int pg_h5_info(const char* filename, const char* path, uint32_t* rank, uint64_t* dims /*[8]*/,
               int32_t* type_class, uint32_t* type_size, int32_t* is_signed);
/* Read converted to dtype into out (capacity in elements). */
int pg_h5_read(const char* filename, const char* path, int32_t dtype, void* out, uint64_t capacity);
/* Newline-separated member names of a group into buf. */
int pg_h5_list(const char* filename, const char* path, char* buf, uint64_t bufsize);

#ifdef __cplusplus
}
#endif
#endif /* PERIGRAIN_IO_H */
