// sph_output.h — VTP files written at output steps without stalling the step stream
// (internal).  Counterpart of writeVTP (src/DataIO/VTPIO.jl:41-98), called by solve! at
// step 0 and at every output step (src/Solve/FluidWallSolve.jl:95,133-136).
//
// Pipeline per file: device-to-device copies of the live fluid's fields into a staging
// slot, ordered on the step stream (so they see exactly the state after the step) ->
// one device-to-host copy of the slot on a separate copy stream -> a host thread that
// orders the particles by upload index and writes the file.  The step stream only
// carries the device-to-device copies; the next steps run while the copy and the file
// write proceed.  Two slots: a third file waits until the first slot is written.
#pragma once

#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdint>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace sph {

// Fluid fields a VTPIO field symbol can name (LiquidParticle.jl:8-64: rho_, p_, c_,
// mass_, gap_; ThermalLiquidParticle adds t_, kappa_, cp_).
enum FluidField { FF_RHO, FF_P, FF_C, FF_MASS, FF_GAP, FF_T, FF_KAPPA, FF_CP, FF_COUNT };

// Device arrays of the sorted fluid state after a step.  The writer copies elements
// [0, n_upper) and the live range [start[cell_lo], start[cell_hi]).
struct FluidSnapshotSrc {
    const void* x;  // double2 (2D) / double4 (3D)
    const void* v;
    const int32_t* id;
    const double* field[FF_COUNT];  // null where the handle has no such field
    const int32_t* start;
    int32_t cell_lo, cell_hi;
    int64_t n_upper;
    // inlet/outlet buffer particles (null bx: none): sorted arrays, live count, capacity;
    // written as the inlet group and the outlet group between the fluid and the walls
    // (FluidInletOutletWallSolve.jl:282), each in ascending order key
    const void* bx;
    const void* bv;
    const double* bfield[5];  // rho p c mass gap
    const int64_t* border;
    const int32_t* bn;
    int64_t bcap;
};

// One wall group (one sph_upload_walls call), host arrays in upload order.
struct WallGroupHost {
    int kind;  // SPH_WALL_*
    int64_t n;
    std::vector<double> x, v, gap, T, kappa;  // x, v: n * dim
};

class VtpWriter {
public:
    VtpWriter() = default;
    VtpWriter(const VtpWriter&) = delete;
    VtpWriter& operator=(const VtpWriter&) = delete;
    ~VtpWriter();

    // Returns an SPH_* status; `err` receives the message on failure.
    int open(int device, int dim, bool thermal, int64_t capacity, const char* dir_path, const char* file_name,
             const char* file_suffix, int step_digit, int n_fields, const char* const* field_symbols,
             const char* const* field_names, const char* wall_time, std::string& err);
    // Wall groups shown after the fluid (group index 2, 3, ...).  Waits for queued files.
    int set_walls(const std::vector<WallGroupHost>& groups, std::string& err);
    // Stage the state for the file of `file_step` at time `time`; returns before the copy.
    int enqueue(cudaStream_t compute, const FluidSnapshotSrc& src, int64_t file_step, double time,
                std::string& err);
    // Wait until every queued file is written; returns the first error met.
    int flush(std::string& err);
    bool is_open() const { return open_; }
    // Path of the file for `file_step` (vtpFileNameAtStep, VTPIO.jl:17-19).
    std::string path_at(int64_t file_step) const;

private:
    struct Slot {
        char* dbuf = nullptr;  // device staging
        char* hbuf = nullptr;  // pinned host copy
        size_t bytes = 0;
        cudaEvent_t staged = nullptr, copied = nullptr;
        bool busy = false;
    };
    struct Job {
        int slot;
        int64_t file_step;
        double time;
        size_t off_x, off_v, off_id, off_range, off_field[FF_COUNT];
        int64_t n_upper;
        bool buffers;  // the file holds the inlet and outlet groups
        size_t off_bx, off_bv, off_bfield[5], off_border, off_bn;
        int64_t bcap;
    };
    void worker();
    int write_file(const Job& job, std::string& err);
    void close();

    bool open_ = false;
    int device_ = 0, dim_ = 2;
    bool thermal_ = false;
    int64_t capacity_ = 0;
    std::string dir_, name_, suffix_, wall_time_;
    int digit_ = 0;
    // per output column: fluid field index (or -1: NaN for the fluid) and name
    std::vector<int> col_fluid_;
    std::vector<std::string> col_symbol_, col_name_;
    std::vector<WallGroupHost> walls_;
    cudaStream_t copy_ = nullptr;
    Slot slot_[2];
    int next_ = 0;
    std::thread thread_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<Job> queue_;
    bool stop_ = false;
    int status_ = 0;
    std::string error_;
};

}  // namespace sph
