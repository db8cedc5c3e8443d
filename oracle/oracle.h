/*
 * oracle.h -- TEST INFRASTRUCTURE: C interface of the CPU restatement of
 * pypybox2d's World.step (oracle.c).  Loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU baseline only.
 */
#ifndef ORACLE_H
#define ORACLE_H

#include <stdint.h>
#include "../include/gb2d.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_world or_world;

/* Build one world from the batch arrays of a scene (world-local copy). */
or_world *or_create(const gb_world_desc *wd, const gb_body *bodies, const gb_fixture *fixtures,
                    const gb_contact *contacts, const int32_t *moves);
void or_destroy(or_world *w);
/* World.step(dt, vel_iters, pos_iters) */
void or_step(or_world *w, double dt, int vel_iters, int pos_iters);

int or_body_count(const or_world *w);
int or_contact_count(const or_world *w);
uint32_t or_world_flags(const or_world *w);
double or_inv_dt0(const or_world *w);
int or_status(const or_world *w);
void or_get_bodies(const or_world *w, gb_body *out);
void or_set_bodies(or_world *w, const gb_body *in);
void or_get_fixtures(const or_world *w, gb_fixture *out);
int or_get_contacts(const or_world *w, gb_contact *out, int cap);
/* Solve the next step's islands in this constraint order (contact-list
 * positions at the time of the island solve). */
void or_set_solver_order(or_world *w, const int *order, int n);
/* Constraint order used by the last step (contact-list positions). */
int or_get_solver_order(const or_world *w, int *out, int cap);
/* out[0..nb): per body the step record of the last step; out[nb..2nb): its
 * island in the solve (smallest non-static body id, -1: none).  Record:
 * position iterations of its
 * island (bits 0-7), TOI position-pass iterations (8-15), TOI events (16-23),
 * parity of its constraints' restitution-bias points and block-solver drops
 * in the island solve (bits 24, 25) and in TOI sub-steps (26, 27) */
void or_get_step_record(const or_world *w, int *out);
void or_clear_status(or_world *w);
/* The world's joints, in World.joints order (replaces any given before);
 * -1 for a bad body index or type. */
int or_set_joints(or_world *w, const gb_joint *joints, int n);
int or_set_controllers(or_world *w, const gb_controller *ctl, int n, const int32_t *bodies, int nbodies);
int or_set_pair_filter(or_world *w, const unsigned char *accept, int n);
/* World.add_joint's filter flag on the contacts between joint j's bodies
 * (world.py:275-281; nothing for a joint with collide_connected). */
void or_flag_joint_contacts(or_world *w, int j);
int or_joint_count(const or_world *w);
void or_get_joints(const or_world *w, gb_joint *out);
/* Solve the next step's joints in this order (world joint indices). */
void or_set_joint_order(or_world *w, const int *order, int n);
/* Joint order of the last step. */
int or_get_joint_order(const or_world *w, int *out, int cap);
long long or_toi_calls(const or_world *w);
long long or_toi_events(const or_world *w);

/* Step every world of a scene n_steps times with `threads` POSIX threads
 * (one world at a time per thread, dynamic assignment).  Bodies of all
 * worlds are written back to `bodies_out` (may be NULL).  Returns the wall
 * time in seconds. */
double or_run_scene(const gb_scene *scene, double dt, int vel_iters, int pos_iters, int n_steps, int threads,
                    gb_body *bodies_out);

/* A persistent batch of worlds for the CPU baseline. */
typedef struct or_batch or_batch;
or_batch *or_batch_create(const gb_scene *scene);
void or_batch_destroy(or_batch *b);
/* n_steps World.step calls on every world, `threads` POSIX threads; wall seconds. */
double or_batch_step(or_batch *b, double dt, int vel_iters, int pos_iters, int n_steps, int threads);
int or_batch_get_bodies(const or_batch *b, int world, gb_body *out);

/* World.ray_cast with a closest-hit callback and World.query_aabb over one
 * world's records (bodies and fixtures world-local; the rays' and queries'
 * world fields are not read). */
void or_ray_cast_records(const gb_body *bodies, const gb_fixture *fixtures, int nf, const gb_ray *rays, int n,
                         gb_ray_hit *hits);
void or_ray_cast_all_records(const gb_body *bodies, const gb_fixture *fixtures, int nf, const gb_ray *rays, int n,
                             gb_ray_hit *hits, int cap, int32_t *counts);
void or_query_aabb_records(const gb_fixture *fixtures, int nf, const gb_aabb_query *qs, int n, int32_t *out, int cap,
                           int32_t *counts);

#ifdef __cplusplus
}
#endif

#endif
