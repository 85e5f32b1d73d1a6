/*
 * config_f32.h -- force-included (nvcc -include) when the reference's CUDA_EA_library kernels
 * are compiled for the oracle's FP32 reference fatbin. TEST INFRASTRUCTURE ONLY.
 *
 * The reference selects `real` with macros in its config.h (CUDA_EA_library/config.h:31-37) and
 * defines GPU_DOUBLE_PRECISION unconditionally; its GPU_SINGLE_PRECISION build needs an edited
 * header. This file pre-empts that header (same include guard) with the same declarations and
 * `real = float`, so the reference sources compile unmodified, in place.
 */
#ifndef __CONFIG_H__
#define __CONFIG_H__
#include <vector>
#include <stdio.h>
#include <stdlib.h>
#include <fstream>
#include <string>
#include <cmath>
#include <time.h>
#include <numeric>
#include <iostream>
#include <iomanip>
using namespace std;

#define TOTAL_RECORD_NUM 20
#define EMIGRATIONS_ISLAND 0
#define EMIGRATIONS_EA 1
#define FLAG_FINISH 2
#define FLAG_DISPLAY_UNIT 3
#define MIN_SUBISLAND_SIZE 4
#define COMPUTING_TIME
#define GPU_SINGLE_PRECISION
typedef float real;

struct Individual { vector<real> elements; real fitness_value; };
typedef vector<Individual> Population;
struct ProblemInfo {
    int dim, function_ID, run_ID, max_base_FEs, seed, running_time, computing_time;
    real max_bound, min_bound;
};
struct NodeInfo { int task_ID, node_ID, node_num, GPU_num, GPU_ID; };
struct IslandInfo {
    int island_size, island_num, interval, migration_size, buffer_capacity;
    real migration_rate;
    int subisland_num;
    string configure_EA, regroup_option, migration_topology, buffer_manage;
};
struct DisplayUnit { real time, communication_percentage, fitness_value; };
#endif
