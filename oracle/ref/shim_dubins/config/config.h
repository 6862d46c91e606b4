/* Golden-vector config: Dubins airplane (the reference's MODEL 2 block of
 * config.h) in the unit cube, dt 0.1, 1..10 steps, speed in [0, 0.3],
 * acceleration in [-0.3, 0.3]; yaw / pitch rates and the pitch bounds come
 * from config_tail.h (DUBINS_AIRPLANE_*). */
#pragma once
#include <math.h>
#define MODEL 2
#define MAX_TREE_SIZE 200000
#define MAX_ITER 300
#define STEP_SIZE 0.1f
#define MAX_PROPAGATION_DURATION 10
#define GOAL_THRESH 0.05f
#define STATE_DIM 6
#define CONTROL_DIM 3
#define SAMPLE_DIM (STATE_DIM + CONTROL_DIM + 1)
#define W_DIM 3
#define C_DIM 2
#define V_DIM 1
#define W_MIN 0.0f
#define W_MAX 1.0f
#define W_SIZE 1.0f
#define C_MIN -M_PI
#define C_MAX M_PI
#define V_MIN 0.0f
#define V_MAX 0.3f
#define A_MIN -0.3f
#define A_MAX 0.3f
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
