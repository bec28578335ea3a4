// frontend.h - host front end compatible with the reference's MCX_userio (fangq/umcx src/umcx.cpp:451-721) and
// with the parameter set-up of MCX_run_simulation (L783-810).
//
// It accepts the same command lines, JSON keys, built-in benchmarks and shape constructs, builds the same label
// volume (including the detector-voxel marking of L605-632), and writes the same .bnii / _detp.jdb files.  The
// photon propagation itself is not here: run.cpp hands the prepared job to the CUDA library.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/umcx_gpu.h"
#include "jsonlite.h"

namespace umcx {

// label volume with the reference's int32 encoding: medium index in the low 31 bits, detector flag in bit 31
struct LabelVolume {
    uint32_t nx = 0, ny = 0, nz = 0;
    std::vector<int32_t> vol;
    void reshape(uint32_t x, uint32_t y, uint32_t z, int32_t value = 0);
    // MCX_volume::index (L128-130): -1 outside
    int64_t index(int ix, int iy, int iz) const;
};

enum class Action { Run, DumpJson, DumpMask, Help };

class UserIO {
public:
    js::Value cfg;
    LabelVolume domain;
    Action action = Action::Run;
    std::string console;  // text the reference would print before exiting (help, --dumpjson)

    // compiled shape constructs of the domain in input order (layers expanded), with the Grid fill value; empty
    // for a JData volume (domain_is_volume), which is decoded into `domain` on the host
    std::vector<umcx_shape_op> shape_ops;
    int32_t grid_fill = 0;
    bool domain_is_volume = false;
    // true: shapes are not painted and detectors not masked on the host; `domain` keeps only the dimensions (and
    // the decoded volume of a JData input) and umcx_gpu_build_labels builds the labels on the GPU
    bool domain_on_device = false;

    // parse a reference command line (argv[0] is the program name), L474-532
    UserIO(int argc, const char* const argv[], bool device_domain = false);
    // JSON string input as MCX_run_json does (L853-856)
    static UserIO from_json(const std::string& json);

    void benchmark(const std::string& name);       // L633-669
    void loadfromfile(const std::string& path);    // L670-672
    void initdomain();                             // L537-604
    void maskdetectors(const js::Value& detectors);  // L605-632
    std::string help_text() const;                 // L533-536

    std::string session_id() const;
    // JNIfTI writers (L673-705)
    void save_volume_f32(const std::vector<float>& data, const uint32_t dim[4], const std::string& file) const;
    void save_volume_i32(const LabelVolume& v, const std::string& file) const;
    void save_detphoton(const std::vector<float>& rows, uint64_t saved, uint64_t detected, int cols,
                        const umcx_sim& sim, const std::string& file) const;

private:
    UserIO() = default;
};

// everything the device kernel needs for one simulation, derived from a parsed configuration (L786-810)
struct Job {
    umcx_sim sim{};
    std::vector<uint8_t> labels;  // uint8: label | 0x80 for detector voxels
    std::vector<float> media;     // [mediumnum][4], mua/mus scaled by unitinmm as at L804
    std::vector<float> detpos;    // [detnum][4]
    umcx_tuning tuning{};         // launch shape from Session.BlockSize / ThreadNum (zeros: the library's default)
    int isnormalized = 1;
    float normalizer_for(double energytotal) const;  // L820
};

// fills a Job from io (throws std::runtime_error on invalid input)
Job make_job(const UserIO& io);

// base64 decoding (for _ArrayZipData_ strings)
std::vector<unsigned char> base64_decode(const std::string& in);

}  // namespace umcx
