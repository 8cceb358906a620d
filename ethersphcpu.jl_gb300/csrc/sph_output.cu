// sph_output.cu — staged VTP output (see sph_output.h).  Host code only.
//
// File layout: VTK XML PolyData with every array in the appended raw block (UInt64
// size headers), the layout src/DataIO/VTPToDataFrame.jl:40-62 reads back (it takes
// the "offset" attribute of every field-data array).  Contents follow writeVTP
// (src/DataIO/VTPIO.jl:41-98):
//   field data  Step (Int64), Time (Float64), WallTime ("yyyy/mm/dd__HH:MM:SS.SS",
//               DataIO.jl:10, in which Julia's Dates reads "SS" as the second both times)
//   point data  Velocity (dim components; NaN for groups without a velocity, :72-80),
//               Type (Int64: 1 for the fluid, then the inlet and outlet particles of
//               the inlet/outlet solve, then the wall groups: 2, 3, ..., :67-69),
//               one Float64 column per field symbol (NaN where the group's particle
//               type has no such field, getParticleFields! :21-38)
//   points      3 components (z = 0 in 2D); one vertex per particle.
// The fluid appears in upload order with deleted particles removed, as the reference's
// particle vector after deleteat! (FluidWallSolve.jl:73-81).
#include "sph_output.h"

#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <limits>

#include "ethersph_gpu.h"

namespace sph {

namespace {

constexpr size_t kAlign = 256;
// order key of an outlet particle (the library's buffer order: bit 62 = outlet)
constexpr int64_t kOutletOrderBit = int64_t(1) << 62;
size_t align_up(size_t v) { return (v + kAlign - 1) / kAlign * kAlign; }

int cuda_err(cudaError_t e, const char* what, std::string& err) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? SPH_ERR_OOM : SPH_ERR_CUDA;
}

#define OUT_CUDA(call, what)                                   \
    do {                                                       \
        cudaError_t _e = (call);                               \
        if (_e != cudaSuccess) return cuda_err(_e, what, err); \
    } while (0)

std::string xml_escape(const std::string& s) {
    std::string o;
    for (char ch : s) {
        switch (ch) {
            case '&': o += "&amp;"; break;
            case '<': o += "&lt;"; break;
            case '>': o += "&gt;"; break;
            case '"': o += "&quot;"; break;
            default: o += ch;
        }
    }
    return o;
}

// Fields that exist on the reference's particle types but are not a scalar state
// (vectors, atomic accumulators): getfield of them cannot fill a Float64 column.
bool is_rejected_symbol(const std::string& s) {
    static const char* bad[] = {"x_vec_", "v_vec_", "normal_vec_", "dv_vec_", "drho_", "sum_kernel_weight_",
                                "sum_weighted_scalar_", "sum_weighted_vector_", "dt_"};
    for (const char* b : bad)
        if (s == b) return true;
    return false;
}

int fluid_field_of(const std::string& s, bool thermal) {
    if (s == "rho_") return FF_RHO;
    if (s == "p_") return FF_P;
    if (s == "c_") return FF_C;
    if (s == "mass_") return FF_MASS;
    if (s == "gap_") return FF_GAP;
    if (thermal && s == "t_") return FF_T;
    if (thermal && s == "kappa_") return FF_KAPPA;
    if (thermal && s == "cp_") return FF_CP;
    return -1;
}

// Column of wall group g for a symbol (WallParticle.jl:8-51): gap_ for every wall,
// t_ and kappa_ for thermostatic walls; null: NaN.
const std::vector<double>* wall_field_of(const WallGroupHost& g, const std::string& s) {
    if (s == "gap_") return &g.gap;
    if (g.kind == SPH_WALL_THERMOSTATIC && s == "t_") return &g.T;
    if (g.kind == SPH_WALL_THERMOSTATIC && s == "kappa_") return &g.kappa;
    return nullptr;
}

std::string wall_time_now() {
    std::time_t t = std::time(nullptr);
    std::tm tm{};
    localtime_r(&t, &tm);
    char buf[64];
    std::snprintf(buf, sizeof buf, "%04d/%02d/%02d__%02d:%02d:%02d.%02d", tm.tm_year + 1900, tm.tm_mon + 1,
                  tm.tm_mday, tm.tm_hour, tm.tm_min, tm.tm_sec, tm.tm_sec);
    return buf;
}

// One appended array: its XML element and its payload.
struct Arr {
    std::string head;  // element text up to offset="
    std::string tail;  // after the offset value
    const char* data;
    uint64_t bytes;
};

}  // namespace

VtpWriter::~VtpWriter() { close(); }

void VtpWriter::close() {
    if (thread_.joinable()) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        thread_.join();
    }
    for (Slot& s : slot_) {
        if (s.dbuf) cudaFree(s.dbuf);
        if (s.hbuf) cudaFreeHost(s.hbuf);
        if (s.staged) cudaEventDestroy(s.staged);
        if (s.copied) cudaEventDestroy(s.copied);
        s = Slot{};
    }
    if (copy_) cudaStreamDestroy(copy_);
    copy_ = nullptr;
    open_ = false;
}

std::string VtpWriter::path_at(int64_t file_step) const {
    std::string num = std::to_string(file_step);
    if (file_step >= 0 && (int)num.size() < digit_) num = std::string(digit_ - num.size(), '0') + num;
    std::string file = name_ + num + suffix_;
    if (dir_.empty()) return file;
    return dir_.back() == '/' ? dir_ + file : dir_ + "/" + file;
}

int VtpWriter::open(int device, int dim, bool thermal, int64_t capacity, const char* dir_path,
                    const char* file_name, const char* file_suffix, int step_digit, int n_fields,
                    const char* const* field_symbols, const char* const* field_names, const char* wall_time,
                    std::string& err) {
    if (!dir_path || !file_name || !file_suffix || n_fields < 0 || (n_fields > 0 && (!field_symbols || !field_names)) ||
        step_digit < 0 || step_digit > 32) {
        err = "sph_output_open: invalid arguments";
        return SPH_ERR_ARG;
    }
    std::vector<int> cols;
    std::vector<std::string> syms, names;
    for (int k = 0; k < n_fields; ++k) {
        if (!field_symbols[k] || !field_names[k]) {
            err = "sph_output_open: null field symbol or name";
            return SPH_ERR_ARG;
        }
        std::string s = field_symbols[k];
        if (!s.empty() && s[0] == ':') s.erase(0, 1);
        if (is_rejected_symbol(s)) {
            err = "sph_output_open: field " + s + " is not a scalar particle state";
            return SPH_ERR_ARG;
        }
        cols.push_back(fluid_field_of(s, thermal));
        syms.push_back(s);
        names.push_back(field_names[k]);
    }
    // assureDirPathExist (DataIO.jl:35-40): one directory level
    if (dir_path[0]) {
        struct stat st{};
        if (stat(dir_path, &st) != 0) {
            if (mkdir(dir_path, 0777) != 0) {
                err = std::string("sph_output_open: cannot create ") + dir_path + ": " + std::strerror(errno);
                return SPH_ERR_IO;
            }
        } else if (!S_ISDIR(st.st_mode)) {
            err = std::string("sph_output_open: ") + dir_path + " is not a directory";
            return SPH_ERR_IO;
        }
    }
    close();
    device_ = device;
    dim_ = dim;
    thermal_ = thermal;
    capacity_ = std::max<int64_t>(capacity, 1);
    dir_ = dir_path;
    name_ = file_name;
    suffix_ = file_suffix;
    digit_ = step_digit;
    wall_time_ = wall_time ? wall_time : "";
    col_fluid_ = cols;
    col_symbol_ = syms;
    col_name_ = names;
    status_ = 0;
    error_.clear();
    stop_ = false;
    next_ = 0;
    // slot size for the whole capacity: x, v, id, live range, fields
    const size_t n = (size_t)capacity_;
    const size_t vb = dim == 2 ? 16 : 32;
    size_t bytes = align_up(n * vb) * 2 + align_up(n * 4) + kAlign;
    for (int c : cols)
        if (c >= 0) bytes += align_up(n * 8);
    OUT_CUDA(cudaStreamCreateWithFlags(&copy_, cudaStreamNonBlocking), "output copy stream");
    for (Slot& s : slot_) {
        OUT_CUDA(cudaMalloc(&s.dbuf, bytes), "output staging (device)");
        OUT_CUDA(cudaMallocHost(&s.hbuf, bytes), "output staging (pinned host)");
        OUT_CUDA(cudaEventCreateWithFlags(&s.staged, cudaEventDisableTiming), "output event");
        OUT_CUDA(cudaEventCreateWithFlags(&s.copied, cudaEventDisableTiming), "output event");
        s.bytes = bytes;
        s.busy = false;
    }
    thread_ = std::thread(&VtpWriter::worker, this);
    open_ = true;
    return SPH_OK;
}

int VtpWriter::set_walls(const std::vector<WallGroupHost>& groups, std::string& err) {
    int rc = flush(err);
    if (rc != SPH_OK) return rc;
    std::lock_guard<std::mutex> lk(mu_);
    walls_ = groups;
    return SPH_OK;
}

int VtpWriter::enqueue(cudaStream_t compute, const FluidSnapshotSrc& src, int64_t file_step, double time,
                       std::string& err) {
    if (!open_) {
        err = "sph_output_write before sph_output_open";
        return SPH_ERR_STATE;
    }
    if (src.n_upper > capacity_) {
        err = "sph_output_write: live fluid exceeds the output capacity";
        return SPH_ERR_ARG;
    }
    Slot& s = slot_[next_];
    {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return !s.busy || stop_; });
        if (status_ != SPH_OK) {
            err = error_;
            return status_;
        }
    }
    const size_t n = (size_t)std::max<int64_t>(src.n_upper, 0);
    const size_t vb = dim_ == 2 ? 16 : 32;
    Job j{};
    j.slot = next_;
    j.file_step = file_step;
    j.time = time;
    j.n_upper = (int64_t)n;
    size_t off = 0;
    j.off_x = off;
    off += align_up(n * vb);
    j.off_v = off;
    off += align_up(n * vb);
    j.off_id = off;
    off += align_up(n * 4);
    j.off_range = off;
    off += kAlign;
    for (int f = 0; f < FF_COUNT; ++f) j.off_field[f] = SIZE_MAX;
    for (int c : col_fluid_) {
        if (c < 0 || j.off_field[c] != SIZE_MAX) continue;
        if (!src.field[c]) {
            err = "sph_output_write: the handle has no such fluid field";
            return SPH_ERR_STATE;
        }
        j.off_field[c] = off;
        off += align_up(n * 8);
    }
    const size_t nb = src.bx ? (size_t)std::max<int64_t>(src.bcap, 0) : 0;
    j.buffers = src.bx != nullptr;
    j.bcap = (int64_t)nb;
    if (src.bx) {  // inlet/outlet buffers: all fields, the order keys, the live count
        j.off_bx = off;
        off += align_up(nb * vb);
        j.off_bv = off;
        off += align_up(nb * vb);
        for (int f = 0; f < 5; ++f) {
            j.off_bfield[f] = off;
            off += align_up(nb * 8);
        }
        j.off_border = off;
        off += align_up(nb * 8);
        j.off_bn = off;
        off += kAlign;
    }
    if (off > s.bytes) {  // a larger state than the slot was sized for: grow it (it is idle)
        if (s.dbuf) cudaFree(s.dbuf);
        if (s.hbuf) cudaFreeHost(s.hbuf);
        s.dbuf = nullptr;
        s.hbuf = nullptr;
        s.bytes = 0;
        OUT_CUDA(cudaMalloc(&s.dbuf, off), "output staging (device)");
        OUT_CUDA(cudaMallocHost(&s.hbuf, off), "output staging (pinned host)");
        s.bytes = off;
    }
    // device-to-device copies, ordered after the steps on the step stream
    if (n > 0) {
        OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_x, src.x, n * vb, cudaMemcpyDeviceToDevice, compute), "stage x");
        OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_v, src.v, n * vb, cudaMemcpyDeviceToDevice, compute), "stage v");
        OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_id, src.id, n * 4, cudaMemcpyDeviceToDevice, compute), "stage id");
        for (int f = 0; f < FF_COUNT; ++f)
            if (j.off_field[f] != SIZE_MAX)
                OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_field[f], src.field[f], n * 8, cudaMemcpyDeviceToDevice,
                                         compute),
                         "stage field");
    }
    OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_range, src.start + src.cell_lo, 4, cudaMemcpyDeviceToDevice, compute),
             "stage range");
    OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_range + 4, src.start + src.cell_hi, 4, cudaMemcpyDeviceToDevice, compute),
             "stage range");
    if (src.bx) {
        if (nb > 0) {
            OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_bx, src.bx, nb * vb, cudaMemcpyDeviceToDevice, compute), "stage");
            OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_bv, src.bv, nb * vb, cudaMemcpyDeviceToDevice, compute), "stage");
            for (int f = 0; f < 5; ++f)
                OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_bfield[f], src.bfield[f], nb * 8, cudaMemcpyDeviceToDevice,
                                         compute),
                         "stage");
            OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_border, src.border, nb * 8, cudaMemcpyDeviceToDevice, compute),
                     "stage");
        }
        OUT_CUDA(cudaMemcpyAsync(s.dbuf + j.off_bn, src.bn, 4, cudaMemcpyDeviceToDevice, compute), "stage");
    }
    OUT_CUDA(cudaEventRecord(s.staged, compute), "output event record");
    // the copy stream takes it from there
    OUT_CUDA(cudaStreamWaitEvent(copy_, s.staged, 0), "output stream wait");
    OUT_CUDA(cudaMemcpyAsync(s.hbuf, s.dbuf, off, cudaMemcpyDeviceToHost, copy_), "output copy to host");
    OUT_CUDA(cudaEventRecord(s.copied, copy_), "output event record");
    {
        std::lock_guard<std::mutex> lk(mu_);
        s.busy = true;
        queue_.push_back(j);
    }
    cv_.notify_all();
    next_ ^= 1;
    return SPH_OK;
}

int VtpWriter::flush(std::string& err) {
    if (!open_) return SPH_OK;
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [&] { return queue_.empty() && !slot_[0].busy && !slot_[1].busy; });
    if (status_ != SPH_OK) {
        err = error_;
        int rc = status_;
        status_ = SPH_OK;
        error_.clear();
        return rc;
    }
    return SPH_OK;
}

void VtpWriter::worker() {
    cudaSetDevice(device_);
    for (;;) {
        Job j{};
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return stop_ || !queue_.empty(); });
            if (queue_.empty()) return;  // stop_ with nothing left
            j = queue_.front();
        }
        std::string err;
        int rc = SPH_OK;
        cudaError_t e = cudaEventSynchronize(slot_[j.slot].copied);
        if (e != cudaSuccess) rc = cuda_err(e, "output copy", err);
        if (rc == SPH_OK) rc = write_file(j, err);
        {
            std::lock_guard<std::mutex> lk(mu_);
            queue_.pop_front();
            slot_[j.slot].busy = false;
            if (rc != SPH_OK && status_ == SPH_OK) {
                status_ = rc;
                error_ = err;
            }
        }
        cv_.notify_all();
    }
}

int VtpWriter::write_file(const Job& j, std::string& err) {
    const char* hb = slot_[j.slot].hbuf;
    const int dim = dim_;
    const size_t vb = dim == 2 ? 16 : 32;
    int32_t b = 0, e = 0;
    std::memcpy(&b, hb + j.off_range, 4);
    std::memcpy(&e, hb + j.off_range + 4, 4);
    if (b < 0 || e < b || e > j.n_upper) {
        err = "output: live range outside the staged particles";
        return SPH_ERR_STATE;
    }
    const int64_t nf = e - b;
    const int32_t* id = (const int32_t*)(hb + j.off_id);
    // upload order: ids ascending (ids are distinct upload indices)
    int32_t max_id = -1;
    for (int64_t k = b; k < e; ++k) max_id = std::max(max_id, id[k]);
    std::vector<int32_t> at((size_t)max_id + 1, -1);
    for (int64_t k = b; k < e; ++k) {
        if (id[k] < 0) {
            err = "output: negative particle id";
            return SPH_ERR_STATE;
        }
        at[(size_t)id[k]] = (int32_t)k;
    }
    std::vector<int32_t> order;
    order.reserve((size_t)nf);
    for (int32_t q = 0; q <= max_id; ++q)
        if (at[(size_t)q] >= 0) order.push_back(at[(size_t)q]);

    // inlet and outlet particles (sorted by order key within each group)
    std::vector<int64_t> inl, outl;
    const double* bx = nullptr;
    const double* bv = nullptr;
    const int64_t* bo = nullptr;
    if (j.buffers) {
        int32_t nb = 0;
        std::memcpy(&nb, hb + j.off_bn, 4);
        if (nb < 0 || nb > j.bcap) {
            err = "output: buffer count outside the staged particles";
            return SPH_ERR_STATE;
        }
        bx = (const double*)(hb + j.off_bx);
        bv = (const double*)(hb + j.off_bv);
        bo = (const int64_t*)(hb + j.off_border);
        for (int64_t k = 0; k < nb; ++k) (bo[k] & kOutletOrderBit ? outl : inl).push_back(k);
        auto by_order = [&](int64_t a, int64_t c) { return bo[a] < bo[c]; };
        std::sort(inl.begin(), inl.end(), by_order);
        std::sort(outl.begin(), outl.end(), by_order);
    }
    const int64_t nbuf = (int64_t)(inl.size() + outl.size());

    int64_t nw = 0;
    for (const WallGroupHost& g : walls_) nw += g.n;
    const int64_t n = nf + nbuf + nw;
    const double nan = std::numeric_limits<double>::quiet_NaN();

    std::vector<double> vel((size_t)n * dim), pts((size_t)n * 3, 0.0);
    std::vector<int64_t> type((size_t)n), conn((size_t)n), offs((size_t)n);
    std::vector<std::vector<double>> cols(col_fluid_.size(), std::vector<double>((size_t)n));
    const double* hx = (const double*)(hb + j.off_x);
    const double* hv = (const double*)(hb + j.off_v);
    const size_t stride = vb / 8;
    for (int64_t q = 0; q < nf; ++q) {
        const size_t k = (size_t)order[(size_t)q];
        for (int a = 0; a < dim; ++a) {
            pts[(size_t)q * 3 + a] = hx[k * stride + a];
            vel[(size_t)q * dim + a] = hv[k * stride + a];
        }
        type[(size_t)q] = 1;
    }
    for (size_t c = 0; c < col_fluid_.size(); ++c) {
        const int f = col_fluid_[c];
        const double* src = f >= 0 ? (const double*)(hb + j.off_field[f]) : nullptr;
        for (int64_t q = 0; q < nf; ++q) cols[c][(size_t)q] = src ? src[order[(size_t)q]] : nan;
    }
    int64_t o = nf;
    int64_t group = 2;
    if (bx) {  // the inlet group, then the outlet group: CommonLiquidParticle vectors
        const std::vector<int64_t>* parts[2] = {&inl, &outl};
        for (const std::vector<int64_t>* part : parts) {
            for (size_t q = 0; q < part->size(); ++q) {
                const size_t k = (size_t)(*part)[q];
                for (int a = 0; a < dim; ++a) {
                    pts[(size_t)(o + q) * 3 + a] = bx[k * stride + a];
                    vel[(size_t)(o + q) * dim + a] = bv[k * stride + a];
                }
                type[(size_t)(o + q)] = group;
            }
            for (size_t c = 0; c < col_fluid_.size(); ++c) {
                const int f = col_fluid_[c];  // rho_ p_ c_ mass_ gap_ exist; thermal fields do not
                const double* src = f >= 0 && f < 5 ? (const double*)(hb + j.off_bfield[f]) : nullptr;
                for (size_t q = 0; q < part->size(); ++q)
                    cols[c][(size_t)(o + q)] = src ? src[(*part)[q]] : nan;
            }
            o += (int64_t)part->size();
            ++group;
        }
    }
    for (const WallGroupHost& g : walls_) {
        const bool has_v = g.kind == SPH_WALL_STATIC_VELOCITY;
        for (int64_t i = 0; i < g.n; ++i) {
            for (int a = 0; a < dim; ++a) {
                pts[(size_t)(o + i) * 3 + a] = g.x[(size_t)i * dim + a];
                vel[(size_t)(o + i) * dim + a] = has_v ? g.v[(size_t)i * dim + a] : nan;
            }
            type[(size_t)(o + i)] = group;
        }
        for (size_t c = 0; c < col_fluid_.size(); ++c) {
            const std::vector<double>* src = wall_field_of(g, col_symbol_[c]);
            for (int64_t i = 0; i < g.n; ++i) cols[c][(size_t)(o + i)] = src ? (*src)[(size_t)i] : nan;
        }
        o += g.n;
        ++group;
    }
    for (int64_t q = 0; q < n; ++q) {
        conn[(size_t)q] = q;
        offs[(size_t)q] = q + 1;
    }
    const int64_t step_val = j.file_step;
    const double time_val = j.time;
    std::string wt = (wall_time_.empty() ? wall_time_now() : wall_time_);
    wt.push_back('\0');

    const std::string N = std::to_string(n);
    std::vector<Arr> arrs;
    auto fd = [&](const char* type, const char* name) {
        return std::string("      <DataArray type=\"") + type + "\" Name=\"" + name +
               "\" NumberOfComponents=\"1\" NumberOfTuples=\"1\" format=\"appended\" offset=\"";
    };
    auto pd = [&](const char* type, const std::string& name, int comps) {
        return std::string("        <DataArray type=\"") + type + "\" Name=\"" + xml_escape(name) +
               "\" NumberOfComponents=\"" + std::to_string(comps) + "\" format=\"appended\" offset=\"";
    };
    const std::string close_el = "\"/>\n";
    std::string pre = "<?xml version=\"1.0\"?>\n"
                      "<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
                      "  <PolyData>\n"
                      "    <FieldData>\n";
    arrs.push_back({pre + fd("Int64", "Step"), close_el, (const char*)&step_val, 8});
    arrs.push_back({fd("Float64", "Time"), close_el, (const char*)&time_val, 8});
    arrs.push_back({fd("String", "WallTime"), close_el, wt.data(), (uint64_t)wt.size()});
    arrs.push_back({"    </FieldData>\n    <Piece NumberOfPoints=\"" + N + "\" NumberOfVerts=\"" + N +
                        "\" NumberOfLines=\"0\" NumberOfStrips=\"0\" NumberOfPolys=\"0\">\n      <PointData>\n" +
                        pd("Float64", "Velocity", dim),
                    close_el, (const char*)vel.data(), (uint64_t)vel.size() * 8});
    arrs.push_back({pd("Int64", "Type", 1), close_el, (const char*)type.data(), (uint64_t)n * 8});
    for (size_t c = 0; c < cols.size(); ++c)
        arrs.push_back({pd("Float64", col_name_[c], 1), close_el, (const char*)cols[c].data(), (uint64_t)n * 8});
    arrs.push_back({"      </PointData>\n      <Points>\n" + pd("Float64", "Points", 3), close_el + "      </Points>\n",
                    (const char*)pts.data(), (uint64_t)n * 24});
    arrs.push_back({"      <Verts>\n" + pd("Int64", "connectivity", 1), close_el, (const char*)conn.data(),
                    (uint64_t)n * 8});
    arrs.push_back({pd("Int64", "offsets", 1),
                    close_el + "      </Verts>\n    </Piece>\n  </PolyData>\n  <AppendedData encoding=\"raw\">\n_",
                    (const char*)offs.data(), (uint64_t)n * 8});

    const std::string path = path_at(j.file_step);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) {
        err = "output: cannot open " + path + ": " + std::strerror(errno);
        return SPH_ERR_IO;
    }
    std::vector<char> iobuf(1 << 22);
    std::setvbuf(f, iobuf.data(), _IOFBF, iobuf.size());
    bool ok = true;
    uint64_t offset = 0;
    for (const Arr& a : arrs) {
        std::string el = a.head + std::to_string(offset) + a.tail;
        ok &= std::fwrite(el.data(), 1, el.size(), f) == el.size();
        offset += 8 + a.bytes;
    }
    for (const Arr& a : arrs) {
        ok &= std::fwrite(&a.bytes, 8, 1, f) == 1;
        if (a.bytes) ok &= std::fwrite(a.data, 1, a.bytes, f) == a.bytes;
    }
    const char* end = "\n  </AppendedData>\n</VTKFile>\n";
    ok &= std::fwrite(end, 1, std::strlen(end), f) == std::strlen(end);
    ok &= std::fclose(f) == 0;
    if (!ok) {
        err = "output: write failed for " + path;
        return SPH_ERR_IO;
    }
    return SPH_OK;
}

}  // namespace sph
