// frontend_check.cpp - host-only driver of the front end (frontend.cpp, jsonlite.cpp) for sanitizer builds.
//
// Reads one input per line from stdin: a JSON array of command-line arguments (argv without the program name), or
// a JSON object taken as MCX_run_json's input.  For each input it parses the command line like the umcx program,
// builds the job a simulation would run (label volume, optical table, detectors, seeds) and writes the files a run
// would write -- the .bnii volume and the _detp.jdb records, filled with synthetic values -- or the --dumpmask volume
// or the --dumpjson/help text.  Prints "ok <summary>" or "error <message>" per input; exits 0 when every input
// was handled (invalid inputs are expected to give "error").
#include <cstdio>
#include <exception>
#include <iostream>
#include <string>
#include <vector>

#include "../../umcx_gb300/csrc/frontend.h"

using umcx::Action;
using umcx::UserIO;
namespace js = umcx::js;

static std::string handle(UserIO& io, int n) {
    const std::string tag = "case" + std::to_string(n);
    if (io.action == Action::Help || io.action == Action::DumpJson) return "text " + std::to_string(io.console.size());
    if (io.action == Action::DumpMask) {
        io.save_volume_i32(io.domain, tag + "_vol.bnii");
        return "mask " + std::to_string(io.domain.vol.size());
    }
    umcx::Job job = umcx::make_job(io);
    const umcx_sim& s = job.sim;
    const size_t nout = 1ULL * s.dim[0] * s.dim[1] * s.dim[2] * s.dim[3];
    if (s.issavevol) {
        std::vector<float> vol(nout);
        for (size_t i = 0; i < nout; i++) vol[i] = static_cast<float>(i % 977) * 0.25f;
        io.save_volume_f32(vol, s.dim, tag + ".bnii");
    }
    if (s.issavedet) {
        const int cols = umcx_detp_columns(&s);
        const uint64_t saved = s.maxdetphotons < 16 ? s.maxdetphotons : 16;
        std::vector<float> rows(saved * static_cast<size_t>(cols));
        for (size_t i = 0; i < rows.size(); i++) rows[i] = static_cast<float>(i) * 0.5f;
        io.save_detphoton(rows, saved, saved + 3, cols, s, tag + "_detp.jdb");
    }
    unsigned labelsum = 0;
    for (uint8_t v : job.labels) labelsum += v;
    return "run " + std::to_string(job.labels.size()) + " " + std::to_string(labelsum) + " " +
           std::to_string(s.mediumnum) + " " + std::to_string(s.detnum);
}

int main() {
    std::string line;
    int n = 0;
    while (std::getline(std::cin, line)) {
        if (line.empty()) continue;
        n++;
        try {
            const js::Value in = js::Value::parse(line);
            if (in.is_array()) {
                std::vector<std::string> args{"umcx"};
                for (size_t i = 0; i < in.size(); i++) args.push_back(in.at(i).as_string());
                std::vector<const char*> argv;
                for (const std::string& a : args) argv.push_back(a.c_str());
                UserIO io(static_cast<int>(argv.size()), argv.data());
                std::printf("ok %s\n", handle(io, n).c_str());
            } else {
                UserIO io = UserIO::from_json(line);
                std::printf("ok %s\n", handle(io, n).c_str());
            }
        } catch (const std::exception& e) {
            std::printf("error %s\n", e.what());
        }
        std::fflush(stdout);
    }
    return 0;
}
