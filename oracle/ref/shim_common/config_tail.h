/* Macros the reference sources reference but the golden-vector configs do not
 * vary (unicycle / Dubins constants, reduction sizes, verbosity). */
#pragma once
#define W_R1_SIZE ((W_MAX - W_MIN) / W_R1_LENGTH)
#define C_R1_SIZE ((C_MAX - C_MIN) / C_R1_LENGTH)
#define V_R1_SIZE ((V_MAX - V_MIN) / V_R1_LENGTH)
#define W_R1_VOL (W_R1_SIZE * W_R1_SIZE * W_R1_SIZE)
#define NUM_R1_REGIONS (W_R1_LENGTH * W_R1_LENGTH * W_R1_LENGTH)
#define NUM_R2_PER_R1 (W_R2_LENGTH * W_R2_LENGTH * W_R2_LENGTH)
#define NUM_R2_REGIONS (NUM_R1_REGIONS * NUM_R2_PER_R1)
#define NUM_R1_REGIONS_KERNEL1 1024
#define NUM_PARTIAL_SUMS 1024
#define EPSILON 1e-2f
#define VERBOSE 0
/* The reference writes these bounds as double expressions (-M_PI / 2, ...),
 * which makes its control draws MIN + u * (MAX - MIN) double arithmetic
 * rounded to float once, while a runtime float config rounds each step.
 * Near steering +-pi/2 one ulp of steering moves tan(steering) by ~1e-4
 * relative, so the golden configs give the same values as float literals
 * (pi/2, pi/4, pi/3 rounded to float): the fixtures then compare the
 * dynamics, not the rounding of a bound. */
#define UNI_MIN_STEERING (-0x1.921fb6p+0f)
#define UNI_MAX_STEERING (0x1.921fb6p+0f)
#define UNI_MIN_DT 0.1f
#define UNI_MAX_DT 2.0f
#define UNI_LENGTH 1.0f
#define DUBINS_AIRPLANE_MIN_PR (-0x1.921fb6p-1f)
#define DUBINS_AIRPLANE_MAX_PR (0x1.921fb6p-1f)
#define DUBINS_AIRPLANE_MIN_YR (-0x1.921fb6p-1f)
#define DUBINS_AIRPLANE_MAX_YR (0x1.921fb6p-1f)
#define DUBINS_AIRPLANE_MIN_PITCH (-0x1.0c1524p+0f)
#define DUBINS_AIRPLANE_MAX_PITCH (0x1.0c1524p+0f)
#define KM 0.03f
