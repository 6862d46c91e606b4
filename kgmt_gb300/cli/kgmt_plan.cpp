// kgmt_plan -- command-line driver in the style of the reference's example
// mains (examples/gpu/main.cu, benchMain.cu, executionTimeMain.cu): load an
// obstacle CSV, copy it to the device, plan, report, and optionally export
// the tree and the goal path as CSV files in the reference's layout
// (KGMT.cu:405-488).  --bench N runs planBench N times (bench runs 0..N-1),
// as benchMain.cu does, writing the per-iteration files under ./Data.
//
//   kgmt_plan --obstacles scene.csv [--model di|quad] [--init x,y,z]
//             [--goal x,y,z] [--seed N] [--capacity N] [--iterations N]
//             [--repeat N] [--bench N] [--out DIR]
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "kgmt.hpp"

static std::vector<float> parse3(const char* s)
{
    std::vector<float> v;
    std::string t(s);
    size_t a = 0;
    while(a <= t.size())
        {
            size_t b = t.find(',', a);
            if(b == std::string::npos) b = t.size();
            if(b > a) v.push_back(std::stof(t.substr(a, b - a)));
            a = b + 1;
        }
    return v;
}

int main(int argc, char** argv)
{
    std::string obstacles, out;
    int model = KGMT_MODEL_DOUBLE_INTEGRATOR;
    std::vector<float> init = {0.05f, 0.05f, 0.05f}, goal = {0.95f, 0.95f, 0.95f};
    long long seed = 1, capacity = -1, iterations = -1, repeat = 1, bench = 0;
    for(int i = 1; i < argc; ++i)
        {
            std::string a = argv[i];
            const char* v = i + 1 < argc ? argv[i + 1] : nullptr;
            if(a == "--obstacles" && v) obstacles = v, ++i;
            else if(a == "--model" && v)
                {
                    const std::string m = v;
                    model = m == "quad" ? KGMT_MODEL_QUADROTOR
                          : m == "dubins" ? KGMT_MODEL_DUBINS_AIRPLANE
                          : m == "unicycle" ? KGMT_MODEL_UNICYCLE : KGMT_MODEL_DOUBLE_INTEGRATOR;
                    ++i;
                }
            else if(a == "--init" && v) init = parse3(v), ++i;
            else if(a == "--goal" && v) goal = parse3(v), ++i;
            else if(a == "--seed" && v) seed = std::atoll(v), ++i;
            else if(a == "--capacity" && v) capacity = std::atoll(v), ++i;
            else if(a == "--iterations" && v) iterations = std::atoll(v), ++i;
            else if(a == "--repeat" && v) repeat = std::atoll(v), ++i;
            else if(a == "--bench" && v) bench = std::atoll(v), ++i;
            else if(a == "--out" && v) out = v, ++i;
            else
                {
                    std::fprintf(stderr, "usage: %s --obstacles scene.csv [--model di|quad|dubins|unicycle] [--init x,y,z] [--goal x,y,z] "
                                         "[--seed N] [--capacity N] [--iterations N] [--repeat N] [--bench N] [--out DIR]\n", argv[0]);
                    return 2;
                }
        }
    try
        {
            kgmt_config cfg = kgmt::default_config(model);
            cfg.seed = (uint64_t)seed;
            if(capacity > 0) cfg.tree_capacity = (uint32_t)capacity;
            if(iterations > 0) cfg.max_iterations = (uint32_t)iterations;
            // the unicycle is planar: rows of four (min x, min y, max x, max y); its
            // --init / --goal third value is the heading (ignored for the goal)
            const int W = model == KGMT_MODEL_UNICYCLE ? 2 : 3;
            std::vector<float> obs = obstacles.empty() ? std::vector<float>() : kgmt::read_obstacles_csv(obstacles, W);
            const uint32_t n = (uint32_t)(obs.size() / (2 * W));
            float* d_obs = nullptr;
            if(n)
                {
                    if(cudaMalloc(&d_obs, obs.size() * sizeof(float)) != cudaSuccess) throw std::runtime_error("cudaMalloc failed");
                    cudaMemcpy(d_obs, obs.data(), obs.size() * sizeof(float), cudaMemcpyHostToDevice);
                }
            const int D = kgmt_sample_dim(model);
            std::vector<float> h_init(D, 0.0f), h_goal(D, 0.0f);
            for(int i = 0; i < 3 && i < (int)init.size(); ++i) h_init[i] = init[i];
            for(int i = 0; i < 3 && i < (int)goal.size(); ++i) h_goal[i] = goal[i];
            kgmt::KGMT planner(cfg);
            for(long long r = 0; r < repeat; ++r)
                {
                    auto t0 = std::chrono::steady_clock::now();
                    planner.plan(h_init.data(), h_goal.data(), d_obs, n);
                    double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
                    const kgmt_result& res = planner.result();
                    std::printf("KGMT execution time: %.6f seconds. Iterations: %u. Tree Size: %u. Status: %d. Goal: %d. Path: %u. "
                                "Cost to goal: %.9g\n",
                                ms * 1e-3, planner.h_itr_, planner.h_treeSize_, res.status, res.goal_index, res.path_len,
                                (double)planner.h_costToGoal_);
                }
            // benchMain.cu:27-32: planBench once per bench run
            for(long long b = 0; b < bench; ++b)
                {
                    planner.planBench(h_init.data(), h_goal.data(), d_obs, n, (int)b);
                    std::printf("KGMT bench %lld: Iterations: %u. Tree Size: %u. Goal: %d\n", b, planner.h_itr_, planner.h_treeSize_,
                                planner.h_pathToGoal_);
                }
            if(!out.empty())
                {
                    std::vector<float> samples, costs;
                    std::vector<int32_t> parents;
                    planner.copy_tree(samples, parents, costs);
                    kgmt::write_csv(out + "/samples.csv", samples.data(), planner.h_treeSize_, D);
                    kgmt::write_csv(out + "/parents.csv", parents.data(), planner.h_treeSize_, 1);
                    kgmt::write_csv(out + "/costs.csv", costs.data(), planner.h_treeSize_, 1);
                    kgmt::write_csv(out + "/controlPathToGoal.csv", planner.h_controlPathToGoal_, planner.h_pathLength_, D);
                }
            if(d_obs) cudaFree(d_obs);
        }
    catch(const std::exception& e)
        {
            std::fprintf(stderr, "%s\n", e.what());
            return 1;
        }
    return 0;
}
