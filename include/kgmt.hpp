// kgmt.hpp -- header-only C++ wrapper over the C ABI (kgmt.h) that keeps the
// reference planner's class surface, so code written against
//   include/planners/Planner.cuh:19-44  (class Planner)
//   include/planners/KGMT.cuh:5-36      (class KGMT : public Planner)
// compiles with a config argument added to the constructor:
//
//   kgmt::KGMT kgmt(cfg);                       // was: KGMT kgmt;
//   kgmt.plan(h_initial, h_goal, d_obstacles, n);
//   kgmt.h_treeSize_, kgmt.h_itr_, kgmt.h_pathToGoal_,
//   kgmt.h_controlPathToGoal_ (goal -> root rows), kgmt.d_treeSamples_ptr_,
//   kgmt.d_treeSamplesParentIdxs_ptr_, kgmt.d_treeSampleCosts_ptr_
//
// Errors are thrown as kgmt::Error (the reference has no error reporting).
#pragma once

#include <cstdint>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
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
// 56-84): fixed notation, 6 decimals, `cols` values per row.
template <typename T>
inline void write_csv(const std::string& path, const T* data, size_t rows, size_t cols)
{
    std::ofstream f(path);
    if(!f) throw std::runtime_error("kgmt: cannot write " + path);
    f.setf(std::ios::fixed);
    f.precision(6);
    for(size_t i = 0; i < rows; ++i)
        {
            for(size_t j = 0; j < cols; ++j)
                {
                    f << data[i * cols + j];
                    if(j + 1 < cols) f << ",";
                }
            f << "\n";
        }
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
    int h_pathToGoal_ = 0;                     // tree index of the goal node, 0 while none
    std::vector<float> h_controlPathToGoal_;   // rows of sample_dim floats, goal -> root

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
    }
    ~KGMT() override { kgmt_destroy(h_); }
    KGMT(const KGMT&) = delete;
    KGMT& operator=(const KGMT&) = delete;

    // KGMT::plan (src/planners/KGMT.cu:41-105): host start/goal rows,
    // caller-owned device obstacle array [n][6] (min xyz, max xyz)
    void plan(float* h_initial, float* h_goal, float* d_obstacles_ptr, unsigned int h_obstaclesCount) override
    {
        check(kgmt_plan(h_, h_initial, h_goal, d_obstacles_ptr, h_obstaclesCount));
        check(kgmt_get_result(h_, &result_));
        h_treeSize_ = result_.tree_size;
        h_itr_ = result_.iterations;
        h_pathToGoal_ = result_.goal_index > 0 ? result_.goal_index : 0;
        const uint32_t D = (uint32_t)kgmt_sample_dim(cfg_.model);
        h_controlPathToGoal_.assign((size_t)result_.path_len * D, 0.0f);
        uint32_t rows = 0;
        check(kgmt_copy_path(h_, h_controlPathToGoal_.data(), result_.path_len, &rows));
        check(kgmt_device_tree(h_, &d_treeSamples_ptr_, &d_treeSamplesParentIdxs_ptr_, &d_treeSampleCosts_ptr_));
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
    kgmt_config cfg_;
    kgmt_planner* h_ = nullptr;
    kgmt_result result_{};
};

}  // namespace kgmt
