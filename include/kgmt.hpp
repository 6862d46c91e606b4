// kgmt.hpp -- header-only C++ wrapper over the C ABI (kgmt.h) that keeps the
// reference planner's class surface, so code written against
//   include/planners/Planner.cuh:19-44  (class Planner)
//   include/planners/KGMT.cuh:5-36      (class KGMT : public Planner)
// compiles with a config argument added to the constructor:
//
//   kgmt::KGMT kgmt(cfg);                       // was: KGMT kgmt;
//   kgmt.plan(h_initial, h_goal, d_obstacles, n);
//   kgmt.planBench(h_initial, h_goal, d_obstacles, n, benchItr);
//   kgmt.h_treeSize_, kgmt.h_itr_, kgmt.h_pathToGoal_, kgmt.h_costToGoal_,
//   kgmt.h_controlPathToGoal_ (float*, goal -> root rows), kgmt.d_treeSamples_ptr_,
//   kgmt.d_treeSamplesParentIdxs_ptr_, kgmt.d_treeSampleCosts_ptr_
//
// Errors are thrown as kgmt::Error (the reference has no error reporting).
#pragma once

#include <cstdint>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <algorithm>
#include <vector>

#include "kgmt.h"

namespace kgmt {

// Obstacle CSV of the reference (include/config/obstacles/*/obstacles.csv,
// read by src/helper/helper.cu:13-39): comma-separated floats, 2 * W per box
// (min corner, max corner; W = workspace_dim, 3, or 2 for the unicycle), any
// line breaks.  Throws on an unreadable file or a count that is not a
// multiple of 2 * W (the reference exits the process).
inline std::vector<float> read_obstacles_csv(const std::string& path, int workspace_dim = 3)
{
    std::ifstream f(path);
    if(!f) throw std::runtime_error("kgmt: cannot open obstacle file " + path);
    std::vector<float> out;
    std::string line;
    while(std::getline(f, line))
        {
            std::stringstream ss(line);
            std::string tok;
            while(std::getline(ss, tok, ','))
                {
                    size_t a = tok.find_first_not_of(" \t\r");
                    if(a == std::string::npos) continue;
                    out.push_back(std::stof(tok.substr(a)));
                }
        }
    const size_t per_box = 2 * (size_t)workspace_dim;
    if(out.size() % per_box != 0)
        throw std::runtime_error("kgmt: obstacle file " + path + " does not hold " + std::to_string(per_box) + " values per box");
    return out;
}

// CSV rows like the reference's writeVectorToCSV (include/helper/helper.cuh:
// 56-84): fixed notation, 6 decimals, `cols` values per row; `append` opens
// the file for appending, as the reference's per-iteration dumps do.
template <typename T>
inline void write_csv(const std::string& path, const T* data, size_t rows, size_t cols, bool append = false)
{
    std::ofstream f(path, append ? std::ios::app : std::ios::trunc);
    if(!f) throw std::runtime_error("kgmt: cannot write " + path);
    f << std::fixed << std::setprecision(6);
    for(size_t i = 0; i < rows; ++i)
        {
            for(size_t j = 0; j < cols; ++j)
                {
                    // bytes (frontier flags) print as numbers, like the reference's bools
                    if constexpr(sizeof(T) == 1) f << (int)data[i * cols + j];
                    else f << data[i * cols + j];
                    if(j + 1 < cols) f << ",";
                }
            f << "\n";
        }
}

// one value appended on its own line, like writeValueToCSV (helper.cuh:94-107)
template <typename T>
inline void append_value_csv(const std::string& path, const T& value)
{
    std::ofstream f(path, std::ios::app);
    if(!f) throw std::runtime_error("kgmt: cannot write " + path);
    if constexpr(std::is_floating_point_v<T>) f << std::fixed << std::setprecision(10);
    f << value << "\n";
}

// The files KGMT::writeDeviceVectorsToCSV (src/planners/KGMT.cu:405-488)
// writes after iteration it.itr of bench run `bench`, under `root`/Data:
// samples<itr>.csv and parents<itr>.csv (all capacity rows), one row per
// iteration of region counters, valid counts, next-frontier flags, repeat
// counts and scores, one line per iteration of frontier size, tree size and
// expanded samples, and the goal -> root path once the goal is reached (its
// path_len rows; the reference writes h_itr_ rows, which cut off the root of
// a path that is one row longer).
inline void write_iteration_csv(const std::string& root, int bench, const kgmt_iteration& it)
{
    namespace fs = std::filesystem;
    const std::string b = std::to_string(bench);
    const std::string data = root.empty() ? std::string("Data") : root + "/Data";
    auto dir = [&](const char* name) {
        const std::string d = data + "/" + name + "/" + name + b;
        fs::create_directories(d);
        return d;
    };
    const std::string itr = std::to_string(it.itr);
    write_csv(dir("Samples") + "/samples" + itr + ".csv", it.samples, it.capacity, it.sample_dim, true);
    write_csv(dir("Parents") + "/parents" + itr + ".csv", it.parents, it.capacity, 1, true);
    write_csv(dir("TotalCountPerVertex") + "/totalCountPerVertex.csv", it.counter, 1, it.regions, true);
    write_csv(dir("ValidCountPerVertex") + "/validCountPerVertex.csv", it.valid, 1, it.regions, true);
    write_csv(dir("Frontier") + "/frontier.csv", it.frontier, 1, it.capacity, true);
    write_csv(dir("FrontierRepeatCount") + "/frontierRepeatCount.csv", it.repeat, 1, it.capacity, true);
    write_csv(dir("VertexScores") + "/vertexScores.csv", it.score, 1, it.regions, true);
    append_value_csv(dir("FrontierSize") + "/frontierSize.csv", it.frontier_size);
    append_value_csv(dir("TreeSize") + "/treeSize.csv", it.tree_size);
    append_value_csv(dir("ExpandedNodes") + "/expandedNodes.csv", it.expanded);
    const std::string path_dir = dir("ControlPathToGoal");
    if(it.goal_index >= 0 && it.path_len) write_csv(path_dir + "/controlPathToGoal.csv", it.path, it.path_len, it.sample_dim, true);
}

class Error : public std::runtime_error {
   public:
    Error(kgmt_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    kgmt_status status;
};

inline void check(kgmt_status s)
{
    if(s != KGMT_OK) throw Error(s, std::string("kgmt: ") + kgmt_last_error());
}

inline kgmt_config default_config(int32_t model = KGMT_MODEL_DOUBLE_INTEGRATOR)
{
    kgmt_config c;
    check(kgmt_config_default(model, &c));
    return c;
}

// Planner base (include/planners/Planner.cuh:19-44)
class Planner {
   public:
    virtual ~Planner() = default;
    virtual void plan(float* h_initial, float* h_goal, float* d_obstacles_ptr, unsigned int h_obstaclesCount) = 0;

    // --- host fields (Planner.cuh:31-34) ---
    unsigned int h_treeSize_ = 0, h_itr_ = 0;
    float h_costToGoal_ = 0.0f;              // the goal node's distance to the goal, 0 while none (the reference never sets it)
    int h_pathToGoal_ = 0;                   // tree index of the goal node, 0 while none
    float* h_controlPathToGoal_ = nullptr;   // rows of sample_dim floats, goal -> root (room for max_iterations + 2 rows)
    unsigned int h_pathLength_ = 0;          // rows of h_controlPathToGoal_ in use

    // --- device fields (Planner.cuh:37-41), valid until the next plan ---
    const float* d_treeSamples_ptr_ = nullptr;
    const int32_t* d_treeSamplesParentIdxs_ptr_ = nullptr;
    const float* d_treeSampleCosts_ptr_ = nullptr;
};

// KGMT (include/planners/KGMT.cuh:5-36)
class KGMT : public Planner {
   public:
    explicit KGMT(const kgmt_config& cfg = default_config(), void* stream = nullptr) : cfg_(cfg)
    {
        check(kgmt_create(&cfg_, stream, &h_));
        // like the reference's new float[SAMPLE_DIM * MAX_ITER] (Planner.cu:22),
        // sized for the longest path a plan of max_iterations can give
        path_.assign(((size_t)cfg_.max_iterations + 2) * (size_t)kgmt_sample_dim(cfg_.model), 0.0f);
        h_controlPathToGoal_ = path_.data();
    }
    ~KGMT() override { kgmt_destroy(h_); }
    KGMT(const KGMT&) = delete;
    KGMT& operator=(const KGMT&) = delete;

    // KGMT::plan (src/planners/KGMT.cu:41-105): host start/goal rows,
    // caller-owned device obstacle array [n][6] (min xyz, max xyz)
    void plan(float* h_initial, float* h_goal, float* d_obstacles_ptr, unsigned int h_obstaclesCount) override
    {
        check(kgmt_plan(h_, h_initial, h_goal, d_obstacles_ptr, h_obstaclesCount));
        read_back();
    }

    // KGMT::planBench (src/planners/KGMT.cu:107-165): the same plan, writing
    // after every iteration the reference's per-iteration CSV files
    // (writeDeviceVectorsToCSV, KGMT.cu:405-488) under Data/ in the working
    // directory (or under data_root/Data), bench run benchItr
    void planBench(float* h_initial, float* h_goal, float* d_obstacles_ptr, unsigned int h_obstaclesCount, int benchItr,
                   const std::string& data_root = std::string())
    {
        struct Ctx {
            const std::string* root;
            int bench;
            std::string error;
        } ctx{&data_root, benchItr, std::string()};
        // the hook runs inside a C call: nothing may be thrown through it
        auto hook = [](const kgmt_iteration* it, void* user) {
            Ctx* c = (Ctx*)user;
            if(!c->error.empty()) return;
            try
                {
                    write_iteration_csv(*c->root, c->bench, *it);
                }
            catch(const std::exception& e)
                {
                    c->error = e.what();
                }
        };
        check(kgmt_plan_traced(h_, h_initial, h_goal, d_obstacles_ptr, h_obstaclesCount, hook, &ctx));
        if(!ctx.error.empty()) throw std::runtime_error(ctx.error);
        read_back();
    }

    const kgmt_result& result() const { return result_; }
    const kgmt_config& config() const { return cfg_; }
    int32_t sample_dim() const { return kgmt_sample_dim(cfg_.model); }

    // host copies of the tree (first h_treeSize_ nodes)
    void copy_tree(std::vector<float>& samples, std::vector<int32_t>& parents, std::vector<float>& costs)
    {
        samples.assign((size_t)h_treeSize_ * sample_dim(), 0.0f);
        parents.assign(h_treeSize_, -1);
        costs.assign(h_treeSize_, 0.0f);
        check(kgmt_copy_tree(h_, samples.data(), parents.data(), costs.data(), h_treeSize_));
    }

   private:
    void read_back()
    {
        check(kgmt_get_result(h_, &result_));
        h_treeSize_ = result_.tree_size;
        h_itr_ = result_.iterations;
        h_pathToGoal_ = result_.goal_index > 0 ? result_.goal_index : 0;
        h_costToGoal_ = result_.goal_cost;
        std::fill(path_.begin(), path_.end(), 0.0f);
        uint32_t rows = 0;
        const uint32_t max_rows = (uint32_t)(path_.size() / (size_t)sample_dim());
        check(kgmt_copy_path(h_, path_.data(), max_rows, &rows));
        h_pathLength_ = rows;
        check(kgmt_device_tree(h_, &d_treeSamples_ptr_, &d_treeSamplesParentIdxs_ptr_, &d_treeSampleCosts_ptr_));
    }

    kgmt_config cfg_;
    kgmt_planner* h_ = nullptr;
    kgmt_result result_{};
    std::vector<float> path_;
};

}  // namespace kgmt
