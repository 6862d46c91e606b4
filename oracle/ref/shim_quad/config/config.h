/* Golden-vector config: 12-D quadrotor in the unit cube, dt 0.02, 1..15
 * steps, thrust in [0,0.3], torques in [-pi,pi], gravity -0.0981, |v| <= 0.3,
 * 16^3 coarse / 4^3 fine workspace-only grid. */
#pragma once
#include <math.h>
#define MODEL 3
#define MAX_TREE_SIZE 2000000
#define MAX_ITER 200
#define STEP_SIZE 0.02f
#define MAX_PROPAGATION_DURATION 15
#define GOAL_THRESH 0.05f
#define STATE_DIM 12
#define CONTROL_DIM 4
#define SAMPLE_DIM (STATE_DIM + CONTROL_DIM + 1)
#define W_DIM 3
#define C_DIM 3
#define V_DIM 3
#define W_MIN 0.0f
#define W_MAX 1.0f
#define W_SIZE 1.0f
#define C_MIN -M_PI
#define C_MAX M_PI
#define V_MIN -0.3f
#define V_MAX 0.3f
#define A_MIN -1.0f
#define A_MAX 1.0f
#define W_R1_LENGTH 16
#define C_R1_LENGTH 1
#define V_R1_LENGTH 1
#define W_R2_LENGTH 4
#define C_R2_LENGTH 1
#define V_R2_LENGTH 1
#define QUAD_MIN_Zc 0.0f
#define QUAD_MAX_Zc 0.3f
#define QUAD_MIN_Lc -M_PI
#define QUAD_MAX_Lc M_PI
#define QUAD_MIN_Mc -M_PI
#define QUAD_MAX_Mc M_PI
#define QUAD_MIN_Nc -M_PI
#define QUAD_MAX_Nc M_PI
#define NU 10e-3f
#define MU 2e-6f
#define IX 1.0f
#define IY 1.0f
#define IZ 2.0f
#define GRAVITY -0.0981f
#define MASS 1.0f
#define MASS_INV 1.0f / MASS
#include "config_tail.h"
