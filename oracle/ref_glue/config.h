/* Hand-written stand-in for the autotools-generated config.h of the reference (test oracle only).
 * The enumerations repeat configure.ac:217-320 of the reference; the physics selection (trajectory
 * type, time flow, Runge-Kutta table) comes from -D flags given by oracle/Makefile, one binary per
 * combination, exactly as a configure run would fix them. */
#ifndef SPX_REF_CONFIG_H
#define SPX_REF_CONFIG_H

#define USE_GSL 1

#define EXEC_SERIAL 0
#define EXEC_PARALLEL 1
#define EXEC_TYPE EXEC_SERIAL

#define TRAJ_FIELDLINE 199
#define TRAJ_LORENTZ 200
#define TRAJ_GUIDING 201
#define TRAJ_GUIDING_SCATT 202
#define TRAJ_GUIDING_DIFF 203
#define TRAJ_GUIDING_DIFF_SCATT 204
#define TRAJ_FOCUSED 205
#define TRAJ_PARKER 206
#define TRAJ_PARKER_SOURCE 207

#define TRAJ_TIME_FLOW_FORWARD 0
#define TRAJ_TIME_FLOW_BACKWARD 1

#define SERVER_SELF 299
#define SERVER_CARTESIAN 300
#define SERVER_BATL 301
#define SERVER_TYPE SERVER_SELF
#define SERVER_INTERP_ORDER -1

#ifndef SPX_REF_TRAJ
#error "SPX_REF_TRAJ must name the trajectory type (e.g. TRAJ_PARKER)"
#endif
#ifndef SPX_REF_FLOW
#error "SPX_REF_FLOW must be TRAJ_TIME_FLOW_FORWARD or TRAJ_TIME_FLOW_BACKWARD"
#endif
#ifndef SPX_REF_RK
#error "SPX_REF_RK must give the Runge-Kutta table number"
#endif

#define TRAJ_TYPE SPX_REF_TRAJ
#define TRAJ_TIME_FLOW SPX_REF_FLOW
#define RK_INTEGRATOR_TYPE SPX_REF_RK

#endif
