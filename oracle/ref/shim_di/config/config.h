/* Golden-vector config: 3-D double integrator in the unit cube, dt 0.05,
 * 1..6 steps, accelerations in [-1,1], |v| <= 0.3, 8^3 coarse / 2^3 fine
 * workspace-only grid (velocity and attitude lengths 1). */
#pragma once
#include <math.h>
#define MODEL 1
#define MAX_TREE_SIZE 100000
#define MAX_ITER 200
#define STEP_SIZE 0.05f
#define MAX_PROPAGATION_DURATION 6
#define GOAL_THRESH 0.05f
#define STATE_DIM 6
#define CONTROL_DIM 3
#define SAMPLE_DIM (STATE_DIM + CONTROL_DIM + 1)
#define W_DIM 3
#define C_DIM 1
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
#define W_R1_LENGTH 8
#define C_R1_LENGTH 1
#define V_R1_LENGTH 1
#define W_R2_LENGTH 2
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
