// frontend.cpp - MCX_userio-compatible front end (fangq/umcx src/umcx.cpp:451-721) and job set-up (L783-810).
//
// Floating-point expressions that decide which voxel gets which label follow the reference's evaluation order
// and this file is compiled with -ffp-contract=off, so rasterised label volumes are identical to the reference's
// on the same input (tests/test_frontend.py compares them with the reference's own --dumpmask output).
#include "frontend.h"

#include "shape_eval.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <atomic>
#include <exception>
#include <mutex>
#include <thread>

#if defined(UMCX_HAVE_ZLIB)
#include <zlib.h>
#endif

namespace umcx {

using js::Value;

static const char* const kOutputTypes = "xfe";  // L57
static const char* const kSourceTypes[] = {"pencil", "isotropic", "cone", "disk", "planar", "fourier"};  // L59
static const char* const kBenchmarks[] = {"cube60",     "cube60b",   "cube60planar", "cubesph60b",
                                          "sphshells",  "spherebox", "skinvessel"};  // L61
enum { kBmCube60, kBmCube60b, kBmCube60planar, kBmCubesph60b, kBmSphshells, kBmSpherebox, kBmSkinvessel, kBmUnknown };

static constexpr int32_t kDetMask = static_cast<int32_t>(0x80000000u);  // L35
static constexpr int32_t kMedMask = 0x7FFFFFFF;                          // L36

void LabelVolume::reshape(uint32_t x, uint32_t y, uint32_t z, int32_t value) {
    nx = x;
    ny = y;
    nz = z;
    vol.assign(static_cast<size_t>(x) * y * z, value);
}

int64_t LabelVolume::index(int ix, int iy, int iz) const {
    // the reference compares 16-bit coordinates against 16-bit sizes (L128-130)
    const int16_t sx = static_cast<int16_t>(ix), sy = static_cast<int16_t>(iy), sz = static_cast<int16_t>(iz);
    if (sx < 0 || sy < 0 || sz < 0 || sx >= static_cast<int16_t>(nx) || sy >= static_cast<int16_t>(ny) ||
        sz >= static_cast<int16_t>(nz))
        return -1;
    return static_cast<int64_t>(sx) * ny * nz + static_cast<int64_t>(sy) * nz + sz;
}

// ------------------------------------------------------------------ command line
struct FlagMap {
    const char* shortf;
    const char* longf;
    const char* pointer;
    char kind;  // 's' string, otherwise parsed as JSON
};
// L454-457
static const FlagMap kFlags[] = {
    {"-n", "--photon", "/Session/Photons", 'f'},       {"-b", "--reflect", "/Session/DoMismatch", 'i'},
    {"-s", "--session", "/Session/ID", 's'},           {"-H", "--maxdetphoton", "/Session/MaxDetPhoton", 'i'},
    {"-u", "--unitinmm", "/Domain/LengthUnit", 'f'},   {"-U", "--normalize", "/Session/DoNormalize", 'i'},
    {"-E", "--seed", "/Session/RNGSeed", 'i'},         {"-O", "--outputtype", "/Session/OutputType", 's'},
    {"-w", "--savedetflag", "/Session/SaveDetFlag", 'i'}, {"-d", "--savedet", "/Session/DoPartialPath", 'i'},
    {"-t", "--thread", "/Session/ThreadNum", 'i'},     {"-T", "--blocksize", "/Session/BlockSize", 'i'},
    {"-G", "--gpuid", "/Session/DeviceID", 'i'},       {"-S", "--save2pt", "/Session/DoSaveVolume", 'i'},
};

std::string UserIO::help_text() const {
    std::string s =
        "/uMCX/ - Portable, massively-parallel physical volumetric ray-tracer (GB300 build)\n\n"
        "Format:\n\tumcx -flag1 value1 -flag2 value2 ...\n\t\tor\n\tumcx inputjson.json\n\tumcx benchmarkname\n\n"
        "Flags:\n"
        "\t-f/--input\tinput json file\n"
        "\t-Q/--bench\t\tbenchmark name\n"
        "\t-n/--photon\tphoton number [1e6]\n"
        "\t-s/--session\toutput name\n"
        "\t-u/--unitinmm\tvoxel size in mm [1]\n"
        "\t-E/--seed\tRNG seed [1648335518]\n"
        "\t-O/--outputtype\t[x]: fluence-rate, f: fluence, e: energy\n"
        "\t-d/--savedet\tSave detected photons [1]\n"
        "\t-S/--save2pt\tSave volumetric output [1]\n"
        "\t-w/--savedetflag\t1:detector-id, 4:partial-path, 16:exit-pos, 32:exit-dir, add to combine [5]\n"
        "\t-U/--normalize\tnormalize output [1]\n"
        "\t-j/--json\tJSON string to overwrite settings\n"
        "\t-t/--thread\tmanual total threads\n"
        "\t-T/--blocksize\tmanual thread-block size [auto]\n"
        "\t-G/--gpuid\tdevice ID [1]\n"
        "\t-b/--reflect\tboundary reflection [1]\n"
        "\t-H/--maxdetphoton\tmaximum saved detected photons [1000000]\n"
        "\t--dumpjson\tdump settings as json\n"
        "\t--dumpmask\tdump domain as binary json\n"
        "\t-h/--help\tprint help\n"
        "\t-N/--net\tbrowse or download simulations from NeuroJSON.io (not available in this program)\n\n"
        "Built-in benchmarks: [\n";
    for (size_t i = 0; i < sizeof(kBenchmarks) / sizeof(kBenchmarks[0]); i++) {
        s += std::string("        \"") + kBenchmarks[i] + "\"";
        s += (i + 1 < sizeof(kBenchmarks) / sizeof(kBenchmarks[0])) ? ",\n" : "\n";
    }
    s += "]\n";
    return s;
}

UserIO::UserIO(int argc, const char* const argv[], bool device_domain) : domain_on_device(device_domain) {
    if (argc < 0) throw std::runtime_error("binary JSON buffer input (MATLAB MEX path) is not supported");
    if (argc <= 1) {  // L480
        action = Action::Help;
        console = help_text();
        return;
    }
    std::vector<std::string> params(argv + 1, argv + argc);
    if (params[0].find('-') == 0) {  // format 1: flags (L484-523)
        for (int i = 1; i < argc;) {
            std::string arg(argv[i++]);
            if ((arg == "-f" || arg == "--input") && i < argc) {
                loadfromfile(argv[i++]);
            } else if (arg == "-h" || arg == "--help") {
                action = Action::Help;
                console = help_text();
                return;
            } else if (arg == "-Q" || arg == "--bench") {
                if (i < argc) {
                    benchmark(argv[i++]);
                } else {
                    action = Action::Help;
                    console = help_text();
                    return;
                }
            } else if ((arg == "-j" || arg == "--json") && i < argc) {
                cfg.update(Value::parse(argv[i++]), true);
            } else if (arg == "-N" || arg == "--net") {
                throw std::runtime_error("-N/--net needs network access, which this program does not provide");
            } else if (arg[0] == '-' && i < argc) {
                for (const FlagMap& f : kFlags) {
                    if (arg == f.shortf || arg == f.longf) {
                        cfg.pointer(f.pointer) =
                            f.kind == 's' ? Value(std::string(argv[i++])) : Value::parse(argv[i++]);
                        break;
                    }
                }
            } else if (!(arg == "--dumpjson" || arg == "--dumpmask")) {
                throw std::runtime_error("incomplete input parameter: " + arg +
                                         "; every -flag/--flag must be followed by a valid value");
            }
        }
    } else if (argc == 2) {  // L517-519
        if (params[0].find('.') == std::string::npos) benchmark(params[0]);
        else loadfromfile(params[0]);
    } else {
        throw std::runtime_error("must use -flag or --flag to use more than 1 input");
    }

    initdomain();

    for (const std::string& p : params) {  // L524-531: --dumpjson wins over --dumpmask
        if (p == "--dumpjson") {
            action = Action::DumpJson;
            console = cfg.dump(2) + "\n";
            return;
        }
    }
    for (const std::string& p : params) {
        if (p == "--dumpmask") {
            action = Action::DumpMask;
            return;
        }
    }
}

UserIO UserIO::from_json(const std::string& json) {
    const char* argv[] = {"", "--json", json.c_str()};
    return UserIO(3, argv);
}

void UserIO::loadfromfile(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open input file " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    cfg = Value::parse(ss.str());
}

std::string UserIO::session_id() const {
    const Value* s = cfg.find("Session");
    const Value* id = s ? s->find("ID") : nullptr;
    return id ? id->as_string() : std::string();
}

// ------------------------------------------------------------------ built-in benchmarks (L633-669)
static Value media_obj(double mua, double mus, double g, double n) {
    Value m = Value::object();
    m["mua"] = mua;
    m["mus"] = mus;
    m["g"] = g;
    m["n"] = n;
    return m;
}
static Value vec3(double a, double b, double c) {
    Value v = Value::array();
    v.push_back(a);
    v.push_back(b);
    v.push_back(c);
    return v;
}
static Value ivec(std::initializer_list<int> xs) {
    Value v = Value::array();
    for (int x : xs) v.push_back(x);
    return v;
}

// the reference writes these fragments as nlohmann `_json` literals, which yield key-sorted objects
static Value sorted_literal(const char* text) {
    Value v = Value::parse(text);
    v.sort_keys();
    return v;
}

void UserIO::benchmark(const std::string& name) {
    int bm = kBmUnknown;
    for (int i = 0; i < kBmUnknown; i++)
        if (name == kBenchmarks[i]) bm = i;
    // the common cube60 set-up: 60^3 grid, label 1 tissue, pencil beam at (29,29,0), four detectors
    Value c = Value::object();
    c["Session"]["ID"] = name;
    c["Session"]["Photons"] = 1000000;
    c["Forward"]["T0"] = 0.0;
    c["Forward"]["T1"] = 5e-9;
    c["Forward"]["Dt"] = 5e-9;
    Value media = Value::array();
    media.push_back(media_obj(0.0, 0.0, 1.0, 1.0));
    media.push_back(media_obj(0.005, 1.0, 0.01, 1.37));
    media.push_back(media_obj(0.002, 5.0, 0.9, 1.0));
    c["Domain"]["Media"] = media;
    c["Domain"]["Dim"] = ivec({60, 60, 60});
    c["Optode"]["Source"]["Type"] = "pencil";
    c["Optode"]["Source"]["Pos"] = vec3(29.0, 29.0, 0.0);
    c["Optode"]["Source"]["Dir"] = vec3(0.0, 0.0, 1.0);
    Value dets = Value::array();
    const int detxy[4][2] = {{29, 19}, {29, 39}, {19, 29}, {39, 29}};
    for (const auto& d : detxy) {
        Value o = Value::object();
        o["Pos"] = ivec({d[0], d[1], 0});
        o["R"] = 1;
        dets.push_back(o);
    }
    c["Optode"]["Detector"] = dets;
    cfg = c;
    cfg["Shapes"] = sorted_literal(R"([{"Grid": {"Tag": 1, "Size": [60, 60, 60]}}])");
    cfg["Session"]["DoMismatch"] = !(bm == kBmCube60 || bm == kBmSkinvessel || bm == kBmSpherebox);

    if (bm == kBmCubesph60b || bm == kBmCube60planar) {
        cfg["Shapes"] = sorted_literal(
            R"([{"Grid": {"Tag": 1, "Size": [60, 60, 60]}}, {"Sphere": {"O": [30, 30, 30], "R": 15, "Tag": 2}}])");
        if (bm == kBmCube60planar) {
            cfg["Optode"]["Source"] = sorted_literal(
                R"({"Type": "planar", "Pos": [10.0, 10.0, -10.0], "Dir": [0.0, 0.0, 1.0], "Param1": [40.0, 0.0, 0.0, 0.0], "Param2": [0.0, 40.0, 0.0, 0.0]})");
        }
    } else if (bm == kBmSkinvessel) {
        cfg["Shapes"] = sorted_literal(
            R"([{"Grid": {"Size": [200, 200, 200], "Tag": 1}}, {"ZLayers": [[1, 20, 1], [21, 32, 4], [33, 200, 3]]}, {"Cylinder": {"Tag": 2, "C0": [0, 100.5, 100.5], "C1": [200, 100.5, 100.5], "R": 20}}])");
        Value fwd = Value::object();
        fwd["T0"] = 0.0;
        fwd["T1"] = 5e-8;
        fwd["Dt"] = 5e-8;
        cfg["Forward"] = fwd;
        cfg["Optode"] = Value::parse(  // an initializer list in the reference: insertion order
            R"({"Source": {"Type": "disk", "Pos": [100, 100, 20], "Dir": [0, 0, 1], "Param1": [60, 0, 0, 0]}})");
        Value dom = Value::object();
        Value m = Value::array();
        m.push_back(media_obj(0.002, 0.0, 1.0, 1.37));
        m.push_back(media_obj(3.564e-05, 1.0, 1.0, 1.37));
        m.push_back(media_obj(23.05426549, 9.398496241, 0.9, 1.37));
        m.push_back(media_obj(0.04584957865, 35.65405549, 0.9, 1.37));
        m.push_back(media_obj(1.657237447, 37.59398496, 0.9, 1.37));
        dom["Media"] = m;
        dom["LengthUnit"] = 0.005;
        dom["Dim"] = ivec({200, 200, 200});
        cfg["Domain"] = dom;
    } else if (bm == kBmSphshells) {
        cfg["Shapes"] = sorted_literal(
            R"([{"Grid": {"Size": [60, 60, 60], "Tag": 1}}, {"Sphere": {"O": [30, 30, 30], "R": 25, "Tag": 2}}, {"Sphere": {"O": [30, 30, 30], "R": 23, "Tag": 3}}, {"Sphere": {"O": [30, 30, 30], "R": 10, "Tag": 4}}])");
        Value m = Value::array();
        m.push_back(media_obj(0.0, 0.0, 1.0, 1.0));
        m.push_back(media_obj(0.02, 7.0, 0.89, 1.37));
        m.push_back(media_obj(0.004, 0.09, 0.89, 1.37));
        m.push_back(media_obj(0.02, 9.0, 0.89, 1.37));
        m.push_back(media_obj(0.05, 0.0, 1.0, 1.37));
        cfg["Domain"]["Media"] = m;
    } else if (bm == kBmSpherebox) {
        cfg["Forward"]["Dt"] = 1e-10;
        Value m = Value::array();
        m.push_back(media_obj(0.0, 0.0, 1.0, 1.0));
        m.push_back(media_obj(0.002, 1.0, 0.01, 1.37));
        m.push_back(media_obj(0.005, 5.0, 0.9, 1.37));
        cfg["Domain"]["Media"] = m;
        cfg["Shapes"] = sorted_literal(
            R"([{"Grid": {"Tag": 1, "Size": [60, 60, 60]}}, {"Sphere": {"O": [30, 30, 30], "R": 10, "Tag": 2}}])");
    } else if (bm >= kBmUnknown) {
        throw std::runtime_error("benchmark " + name + " is not found");
    }
}

// ------------------------------------------------------------------ domain rasteriser (L458-473, L537-604)
struct P3 {
    float x, y, z;
};

// A shape construct compiled once into plain floats; evaluated per voxel centre with the reference's float
// expressions (L458-473).  A missing key throws where the reference's lookup would: for a value that every voxel
// reads, at the first voxel; for one read only inside the shape (the tag, the Box extent), at the first voxel that
// reaches it.  0 = not inside (the reference returns int quiet_NaN, i.e. 0).
struct OptF {
    float v = 0.f;
    bool ok = false;
};
static OptF opt_num(const Value& o, const char* key, size_t i) {
    OptF r;
    const Value* a = o.find(key);
    if (a && a->is_array() && i < a->size() && a->at(i).is_number()) {
        r.v = a->at(i).as_float();
        r.ok = true;
    }
    return r;
}
static OptF opt_scalar(const Value& v) {
    OptF r;
    if (v.is_number() || v.is_bool()) {
        r.v = v.as_float();
        r.ok = true;
    }
    return r;
}
[[noreturn]] static void missing_number() { throw js::type_error("type must be number, but is null"); }
static float need(const OptF& f) {
    if (!f.ok) missing_number();
    return f.v;
}

// Compiles one shape construct into device-evaluable ops (shape_eval.h), appended to *ops: a layers construct
// gives one op per layer, in order.  Values every voxel reads are required here (the reference throws at the first
// voxel); values read only inside a shape (the tag, the Box extent, a layer's upper bound) are recorded as present
// or not and reported where a voxel reaches them.  Returns false for a key that is not a shape.
static bool compile_shape(const std::string& key, const Value& body, std::vector<umcx_shape_op>* ops) {
    auto read_tag = [&](const Value& v, umcx_shape_op* op) {
        const Value* t = v.find("Tag");
        if (t && (t->is_number() || t->is_bool())) {
            op->tag = t->as_int();
            op->present |= UMCX_SHAPE_HAS_TAG;
        }
    };
    umcx_shape_op op;
    std::memset(&op, 0, sizeof(op));
    if (key == "Sphere") {
        op.kind = UMCX_SHAPE_SPHERE;
        for (int k = 0; k < 3; k++) op.f[k] = need(opt_num(body, "O", static_cast<size_t>(k)));
        op.f[3] = need(opt_scalar(body.contains("R") ? body.at("R") : Value()));
        read_tag(body, &op);
        ops->push_back(op);
    } else if (key == "Box") {
        // the reference reads a key spelled "Sip.ze" and compares p.x three times (L460)
        op.kind = UMCX_SHAPE_BOX;
        for (int k = 0; k < 3; k++) op.f[k] = need(opt_num(body, "O", static_cast<size_t>(k)));
        for (int k = 0; k < 3; k++) {
            const OptF sz = opt_num(body, "Sip.ze", static_cast<size_t>(k));
            op.f[3 + k] = sz.v;
            if (sz.ok) op.present |= UMCX_SHAPE_HAS_SIZE0 << k;
        }
        read_tag(body, &op);
        ops->push_back(op);
    } else if (key == "XLayers" || key == "YLayers" || key == "ZLayers") {
        const int kind = key[0] == 'X' ? UMCX_SHAPE_XLAYER : (key[0] == 'Y' ? UMCX_SHAPE_YLAYER : UMCX_SHAPE_ZLAYER);
        for (const Value& layer : body.items()) {
            umcx_shape_op L;
            std::memset(&L, 0, sizeof(L));
            L.kind = kind;
            if (!layer.is_array()) missing_number();
            const OptF lo = layer.size() > 0 ? opt_scalar(layer.at(0)) : OptF();
            const OptF hi = layer.size() > 1 ? opt_scalar(layer.at(1)) : OptF();
            L.f[0] = need(lo);
            L.f[1] = hi.v;
            if (hi.ok) L.present |= UMCX_SHAPE_HAS_HI;
            if (layer.size() > 2 && (layer.at(2).is_number() || layer.at(2).is_bool())) {
                L.tag = layer.at(2).as_int();
                L.present |= UMCX_SHAPE_HAS_TAG;
            }
            ops->push_back(L);
        }
    } else if (key == "Cylinder") {
        op.kind = UMCX_SHAPE_CYLINDER;
        float c0[3], c1[3];
        for (int k = 0; k < 3; k++) {
            c0[k] = need(opt_num(body, "C0", static_cast<size_t>(k)));
            c1[k] = need(opt_num(body, "C1", static_cast<size_t>(k)));
        }
        const float ax = c1[0] - c0[0], ay = c1[1] - c0[1], az = c1[2] - c0[2];
        const float d0 = ax * ax + ay * ay + az * az;
        for (int k = 0; k < 3; k++) op.f[k] = c0[k];
        op.f[3] = ax / sqrtf(d0);
        op.f[4] = ay / sqrtf(d0);
        op.f[5] = az / sqrtf(d0);
        op.f[6] = d0;
        op.f[7] = need(opt_scalar(body.contains("R") ? body.at("R") : Value()));
        read_tag(body, &op);
        ops->push_back(op);
    } else {
        return false;
    }
    return true;
}

std::vector<unsigned char> base64_decode(const std::string& in) {
    static int8_t lut[256];
    static bool init = false;
    if (!init) {
        std::memset(lut, -1, sizeof(lut));
        const char* a = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
        for (int i = 0; i < 64; i++) lut[static_cast<unsigned char>(a[i])] = static_cast<int8_t>(i);
        init = true;
    }
    std::vector<unsigned char> out;
    out.reserve(in.size() * 3 / 4);
    uint32_t acc = 0;
    int bits = 0;
    for (unsigned char c : in) {
        if (c == '=') break;
        int8_t v = lut[c];
        if (v < 0) continue;  // skip whitespace / line breaks
        acc = (acc << 6) | static_cast<uint32_t>(v);
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back(static_cast<unsigned char>((acc >> bits) & 0xFF));
        }
    }
    return out;
}

static std::vector<unsigned char> inflate_bytes(const std::vector<unsigned char>& in, bool gzip) {
#if defined(UMCX_HAVE_ZLIB)
    z_stream zs;
    std::memset(&zs, 0, sizeof(zs));
    if (inflateInit2(&zs, gzip ? 15 + 16 : 15) != Z_OK) throw std::runtime_error("zlib: inflateInit failed");
    std::vector<unsigned char> out;
    std::vector<unsigned char> buf(1 << 20);
    zs.next_in = const_cast<unsigned char*>(in.data());
    zs.avail_in = static_cast<uInt>(in.size());
    int rc;
    do {
        zs.next_out = buf.data();
        zs.avail_out = static_cast<uInt>(buf.size());
        rc = inflate(&zs, Z_NO_FLUSH);
        if (rc != Z_OK && rc != Z_STREAM_END) {
            inflateEnd(&zs);
            throw std::runtime_error("zlib: corrupt compressed volume data");
        }
        out.insert(out.end(), buf.data(), buf.data() + (buf.size() - zs.avail_out));
    } while (rc != Z_STREAM_END);
    inflateEnd(&zs);
    return out;
#else
    (void)in;
    (void)gzip;
    throw std::runtime_error("_ArrayZipData_ volumes need zlib, which this library was compiled without");
#endif
}

template <class T>
static void copy_cast(const std::vector<unsigned char>& raw, std::vector<int32_t>& dst) {
    const size_t n = dst.size();
    if (raw.size() < n * sizeof(T)) throw std::runtime_error("_ArrayZipData_ holds fewer elements than _ArraySize_");
    for (size_t i = 0; i < n; i++) {
        T v;
        std::memcpy(&v, raw.data() + i * sizeof(T), sizeof(T));
        dst[i] = static_cast<int32_t>(v);
    }
}

void UserIO::initdomain() {
    const Value& dim = cfg.at("Domain").at("Dim");
    uint32_t nx = static_cast<uint32_t>(dim.at(0).as_uint64()), ny = static_cast<uint32_t>(dim.at(1).as_uint64()),
             nz = static_cast<uint32_t>(dim.at(2).as_uint64());
    shape_ops.clear();
    grid_fill = 0;
    domain_is_volume = false;
    const Value* shapes = cfg.find("Shapes");
    if (shapes && shapes->contains("_ArraySize_")) {  // JData volume (L571-598): decoded on the host
        domain_is_volume = true;
        const Value& sz = shapes->at("_ArraySize_");
        domain.reshape(static_cast<uint32_t>(sz.at(0).as_uint64()), static_cast<uint32_t>(sz.at(1).as_uint64()),
                       static_cast<uint32_t>(sz.at(2).as_uint64()));
        const std::string dtype = shapes->value("_ArrayType_", std::string("int32"));
        if (const Value* data = shapes->find("_ArrayData_")) {
            const size_t n = domain.vol.size();
            if (data->size() < n) throw std::runtime_error("_ArrayData_ holds fewer elements than _ArraySize_");
            for (size_t i = 0; i < n; i++) domain.vol[i] = static_cast<int32_t>(data->at(i).as_int64());
        } else if (const Value* zdata = shapes->find("_ArrayZipData_")) {
            std::vector<unsigned char> zbuf;
            if (zdata->is_string()) {
                zbuf = base64_decode(zdata->as_string());
            } else {
                for (const Value& b : zdata->items()) zbuf.push_back(static_cast<unsigned char>(b.as_uint64()));
            }
            const bool gzip = shapes->value("_ArrayZipType_", std::string("zlib")) == "gzip";
            std::vector<unsigned char> raw = inflate_bytes(zbuf, gzip);
            if (dtype == "uint8") copy_cast<uint8_t>(raw, domain.vol);
            else if (dtype == "int8") copy_cast<int8_t>(raw, domain.vol);
            else if (dtype == "uint16") copy_cast<uint16_t>(raw, domain.vol);
            else if (dtype == "int16") copy_cast<int16_t>(raw, domain.vol);
            else if (dtype == "uint32") copy_cast<uint32_t>(raw, domain.vol);
            else copy_cast<int32_t>(raw, domain.vol);
        }
    } else {
        // shape constructs (L537-570), compiled into ops one construct at a time and, unless the domain is built on
        // the device (umcx_gpu_build_labels), painted on host threads before the next construct is read
        const Value* first = shapes ? (shapes->is_array() ? &shapes->at(0) : shapes) : nullptr;
        if (first) {
            if (const Value* grid = first->find("Grid")) {
                const Value& sz = grid->at("Size");
                nx = static_cast<uint32_t>(sz.at(0).as_uint64());
                ny = static_cast<uint32_t>(sz.at(1).as_uint64());
                nz = static_cast<uint32_t>(sz.at(2).as_uint64());
                grid_fill = grid->at("Tag").as_int();
            }
        }
        if (domain_on_device) {
            domain.nx = nx;
            domain.ny = ny;
            domain.nz = nz;
            domain.vol.clear();
        } else {
            domain.reshape(nx, ny, nz, grid_fill);
        }
        auto paint = [&](size_t op_begin, size_t op_end) {
            // z-slabs on host threads (every voxel is written by exactly one thread)
            std::atomic<uint32_t> nextz{0};
            std::atomic<bool> missing{false};
            auto slabs = [&]() {
                bool miss = false;
                for (uint32_t z; !miss && (z = nextz.fetch_add(1)) < domain.nz;)
                    for (uint32_t y = 0; y < domain.ny; y++)
                        for (uint32_t x = 0; x < domain.nx; x++) {
                            const int64_t idx = domain.index(static_cast<int>(x), static_cast<int>(y), static_cast<int>(z));
                            const float px = x + 0.5f, py = y + 0.5f, pz = z + 0.5f;
                            for (size_t k = op_begin; k < op_end; k++) {
                                const int label = umcx_shape::eval_op(shape_ops[k], px, py, pz, &miss);
                                if (label) domain.vol[static_cast<size_t>(idx)] = label;  // MCX_volume::mask, L138-140
                            }
                        }
                if (miss) {
                    missing.store(true);
                    nextz.store(domain.nz);
                }
            };
            const size_t nvox = static_cast<size_t>(domain.nx) * domain.ny * domain.nz;
            unsigned nthr = std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
            if (nvox < (1u << 16)) nthr = 1;
            std::vector<std::thread> pool;
            for (unsigned t = 1; t < nthr; t++) pool.emplace_back(slabs);
            slabs();
            for (auto& th : pool) th.join();
            if (missing.load()) missing_number();
        };
        if (shapes) {
            std::vector<const Value*> objs;
            if (shapes->is_array()) {
                for (const Value& o : shapes->items()) objs.push_back(&o);
            } else {
                for (const auto& m : shapes->members()) objs.push_back(&m.second);
            }
            for (const Value* obj : objs) {
                const std::string key = obj->is_object() && !obj->empty() ? obj->front_member().first : std::string();
                const size_t before = shape_ops.size();
                if (compile_shape(key, obj->front_member().second, &shape_ops)) {
                    if (!domain_on_device) paint(before, shape_ops.size());
                } else if (!(key == "Name" || key == "Grid" || key == "Origin")) {
                    throw std::runtime_error("shape construct" + key + " is not supported");
                }
            }
        }
    }
    if (domain_on_device) return;  // detectors are masked by the device label builder
    const Value* optode = cfg.find("Optode");
    if (optode && optode->contains("Detector")) maskdetectors(optode->at("Detector"));
}

void UserIO::maskdetectors(const Value& detectors) {
    // 26 neighbour offsets in the reference's order (L606)
    static const int8_t nb[26][3] = {{-1, -1, -1}, {0, -1, -1}, {1, -1, -1}, {-1, 0, -1}, {0, 0, -1}, {1, 0, -1},
                                     {-1, 1, -1},  {0, 1, -1},  {1, 1, -1},  {-1, -1, 0}, {0, -1, 0}, {1, -1, 0},
                                     {-1, 0, 0},   {1, 0, 0},   {-1, 1, 0},  {0, 1, 0},   {1, 1, 0},  {-1, -1, 1},
                                     {0, -1, 1},   {1, -1, 1},  {-1, 0, 1},  {0, 0, 1},   {1, 0, 1},  {-1, 1, 1},
                                     {0, 1, 1},    {1, 1, 1}};
    const int64_t total = static_cast<int64_t>(domain.vol.size());
    auto label_at = [&](int64_t i) -> int32_t {
        // neighbours beyond the array (undefined in the reference) count as background
        return (i >= 0 && i < total) ? domain.vol[static_cast<size_t>(i)] : 0;
    };
    for (const Value& det : detectors.items()) {
        const float radius = det.at("R").as_float();
        const float dx = det.at("Pos").at(0).as_float(), dy = det.at("Pos").at(1).as_float(),
                    dz = det.at("Pos").at(2).as_float();
        for (float iz = -radius - 1.f + dz; iz <= radius + 1.f + dz; iz += 0.5f)
            for (float iy = -radius - 1.f + dy; iy <= radius + 1.f + dy; iy += 0.5f)
                for (float ix = -radius - 1.f + dx; ix <= radius + 1.f + dx; ix += 0.5f) {
                    const int16_t sx = static_cast<int16_t>(ix), sy = static_cast<int16_t>(iy), sz = static_cast<int16_t>(iz);
                    const int64_t idx = domain.index(sx, sy, sz);
                    if (idx < 0 ||
                        (ix - dx) * (ix - dx) + (iy - dy) * (iy - dy) + (iz - dz) * (iz - dz) >
                            (radius + 1.f) * (radius + 1.f) ||
                        (domain.vol[static_cast<size_t>(idx)] & kMedMask) == 0)
                        continue;
                    if (static_cast<int>(sx) * sy * sz == 0 || sx == static_cast<int16_t>(domain.nx) ||
                        sy == static_cast<int16_t>(domain.ny) || sz == static_cast<int16_t>(domain.nz)) {
                        domain.vol[static_cast<size_t>(idx)] |= kDetMask;
                    } else {
                        for (int k = 0; k < 26; k++) {
                            // the reference offsets by index(dx,dy,dz), which is -1 whenever a component is negative
                            const int64_t off = domain.index(nb[k][0], nb[k][1], nb[k][2]);
                            if ((label_at(idx + off) & kMedMask) == 0) {
                                domain.vol[static_cast<size_t>(idx)] |= kDetMask;
                                break;
                            }
                        }
                    }
                }
    }
}

// ------------------------------------------------------------------ writers (L673-705)
static void write_file(const std::string& path, const std::string& bytes) {
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot write output file " + path);
    f.write(bytes.data(), static_cast<std::streamsize>(bytes.size()));
}

static Value dims4(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    Value v = Value::array();
    v.push_back(a);
    v.push_back(b);
    v.push_back(c);
    v.push_back(d);
    return v;
}

void UserIO::save_volume_f32(const std::vector<float>& data, const uint32_t dim[4], const std::string& file) const {
    Value f = Value::object();
    f["NIFTIHeader"]["Dim"] = dims4(dim[0], dim[1], dim[2], dim[3]);
    Value nd = Value::object();
    nd["_ArraySize_"] = dims4(dim[0], dim[1], dim[2], dim[3]);
    nd["_ArrayType_"] = "single";
    nd["_ArrayData_"] = Value::packed('d', data.data(), data.size());
    f["NIFTIData"] = nd;
    std::string out;
    f.to_bjdata(out);
    write_file(file, out);
}

void UserIO::save_volume_i32(const LabelVolume& v, const std::string& file) const {
    Value f = Value::object();
    f["NIFTIHeader"]["Dim"] = dims4(v.nx, v.ny, v.nz, 1);
    Value nd = Value::object();
    nd["_ArraySize_"] = dims4(v.nx, v.ny, v.nz, 1);
    nd["_ArrayType_"] = "int32";
    nd["_ArrayData_"] = Value::packed('l', v.vol.data(), v.vol.size());
    f["NIFTIData"] = nd;
    std::string out;
    f.to_bjdata(out);
    write_file(file, out);
}

void UserIO::save_detphoton(const std::vector<float>& rows, uint64_t saved, uint64_t detected, int cols,
                            const umcx_sim& sim, const std::string& file) const {
    Value info = Value::object();
    info["Version"] = 1;
    info["MediaNum"] = sim.mediumnum;
    info["DetNum"] = sim.detnum;
    info["ColumnNum"] = cols;
    info["TotalPhoton"] = cols;  // the reference stores the column count here (L689)
    info["DetectedPhoton"] = static_cast<uint32_t>(detected);
    info["SavedPhoton"] = static_cast<uint32_t>(saved);
    info["LengthUnit"] = static_cast<double>(sim.unitinmm);
    Value raw = Value::object();
    Value size = Value::array();
    size.push_back(static_cast<uint32_t>(saved));
    size.push_back(Value::integer(cols));
    raw["_ArraySize_"] = size;
    raw["_ArrayType_"] = "single";
    raw["_ArrayData_"] = Value::packed('d', rows.data(), static_cast<size_t>(saved) * static_cast<size_t>(cols));
    Value top = Value::object();
    top["MCXData"]["Info"] = info;
    top["MCXData"]["PhotonRawData"] = raw;
    std::string out;
    top.to_bjdata(out);
    write_file(file, out);
}

// ------------------------------------------------------------------ job set-up (L786-810)
float Job::normalizer_for(double energytotal) const {
    if (sim.outputtype == UMCX_OUT_ENERGY) return static_cast<float>(1.f / energytotal);
    if (sim.outputtype == UMCX_OUT_FLUENCE_RATE)
        return static_cast<float>(sim.rtstep / (energytotal * sim.unitinmm * sim.unitinmm));
    return static_cast<float>(1.f / (energytotal * sim.unitinmm * sim.unitinmm));
}

Job make_job(const UserIO& io) {
    const Value& cfg = io.cfg;
    Job job;
    umcx_sim& s = job.sim;
    std::memset(&s, 0, sizeof(s));
    const Value& session = cfg.contains("Session") ? cfg.at("Session") : Value::object();
    const Value& fwd = cfg.at("Forward");
    const Value& domain = cfg.at("Domain");
    const Value& source = cfg.at("Optode").at("Source");
    const float t0 = fwd.at("T0").as_float(), t1 = fwd.at("T1").as_float(), dt = fwd.at("Dt").as_float();
    s.tstart = t0;
    s.tend = t1;
    s.rtstep = 1.f / dt;
    s.unitinmm = static_cast<float>(domain.value("LengthUnit", 1.0));
    const int maxgate = static_cast<int>((t1 - t0) / dt + 0.5f);
    if (maxgate < 1 || maxgate > UMCX_MAX_GATES)
        throw std::runtime_error("invalid time gates: (T1-T0)/Dt must give between 1 and 65535 gates");
    s.isreflect = static_cast<int32_t>(session.value_int("DoMismatch", 1));
    job.isnormalized = static_cast<int>(session.value_int("DoNormalize", 1));
    s.issavevol = static_cast<int32_t>(session.value_int("DoSaveVolume", 1));
    s.issavedet = static_cast<int32_t>(session.value_int("DoPartialPath", 1));
    s.savedetflag = static_cast<int32_t>(session.value_int("SaveDetFlag", UMCX_DET_ID + UMCX_DET_PPATH));
    const Value& media = domain.at("Media");
    s.mediumnum = static_cast<int32_t>(media.size());
    if (s.mediumnum < 1 || s.mediumnum > UMCX_MAX_MEDIA)
        throw std::runtime_error("Domain.Media must list between 1 and 128 media");
    const std::string otype = session.value("OutputType", std::string("x"));
    const char* hit = otype.empty() ? nullptr : std::strchr(kOutputTypes, otype[0]);
    s.outputtype = hit ? static_cast<int32_t>(hit - kOutputTypes) : -1;
    const Value* optode = cfg.find("Optode");
    s.detnum = (optode && optode->contains("Detector")) ? static_cast<int32_t>(optode->at("Detector").size()) : 0;
    if (s.detnum > UMCX_MAX_DET) throw std::runtime_error("at most 64 detectors are supported");
    s.maxdetphotons = static_cast<uint32_t>(session.value_int("MaxDetPhoton", 1000000));
    if (!s.issavedet) s.maxdetphotons = 0;  // MCX_detect, L155
    const std::string stype = source.value("Type", std::string("pencil"));
    s.srctype = 6;  // unknown type: launched like a pencil beam (L225-259)
    for (int i = 0; i < 6; i++)
        if (stype == kSourceTypes[i]) s.srctype = i;
    for (int k = 0; k < 4; k++) {
        s.srcparam1[k] = source.contains("Param1") ? source.at("Param1").at(static_cast<size_t>(k)).as_float() : 0.f;
        s.srcparam2[k] = source.contains("Param2") ? source.at("Param2").at(static_cast<size_t>(k)).as_float() : 0.f;
    }
    for (int k = 0; k < 3; k++) {
        s.srcpos[k] = source.at("Pos").at(static_cast<size_t>(k)).as_float();
        s.srcdir[k] = source.at("Dir").at(static_cast<size_t>(k)).as_float();
    }
    s.srcpos[3] = 1.f;
    s.srcdir[3] = 0.f;
    s.dim[0] = io.domain.nx;
    s.dim[1] = io.domain.ny;
    s.dim[2] = io.domain.nz;
    s.dim[3] = static_cast<uint32_t>(maxgate);
    if (io.domain.nx == 0 || io.domain.ny == 0 || io.domain.nz == 0 || io.domain.nx > 32767 || io.domain.ny > 32767 ||
        io.domain.nz > 32767)
        throw std::runtime_error("domain dimensions must be between 1 and 32767");

    // Photons: read with get<uint64_t> at L813 (required), seeds at L724-727
    const Value* photons = session.find("Photons");
    if (!photons) throw js::type_error("type must be number, but is null");
    s.nphoton = photons->as_uint64();
    s.photon_offset = 0;
    int32_t rngseed = 1648335518;
    if (const Value* sv = session.find("RNGSeed")) rngseed = sv->as_int();
    umcx_seeds_from_rngseed(rngseed, s.seeds);

    // launch shape (L739-741): when BlockSize or ThreadNum is given, CTAs of BlockSize threads (default 64) and
    // ThreadNum / BlockSize of them (ThreadNum default 100000), as the reference's GPU build launches; the block is
    // rounded up to whole warps because the kernels vote per warp.  Without either key the library's own
    // persistent launch (one wave of resident CTAs) is used.
    if (session.contains("BlockSize") || session.contains("ThreadNum")) {
        const int64_t bs = session.value_int("BlockSize", 64), tn = session.value_int("ThreadNum", 100000);
        if (bs < 1 || bs > 1024) throw std::runtime_error("BlockSize must be between 1 and 1024");
        if (tn < 1) throw std::runtime_error("ThreadNum must be positive");
        job.tuning.block_size = static_cast<int32_t>((bs + 31) / 32 * 32);
        const int64_t grid = tn / bs;
        job.tuning.grid_size = static_cast<int32_t>(grid < 1 ? 1 : (grid > (1 << 24) ? (1 << 24) : grid));
    }

    // media table (L800-806)
    job.media.resize(static_cast<size_t>(s.mediumnum) * 4);
    for (int i = 0; i < s.mediumnum; i++) {
        const Value& m = media.at(static_cast<size_t>(i));
        float* d = &job.media[static_cast<size_t>(i) * 4];
        if (m.is_array()) {
            if (m.size() < 4) throw std::runtime_error("a medium given as an array needs [mua, mus, g, n]");
            for (int k = 0; k < 4; k++) d[k] = m.at(static_cast<size_t>(k)).as_float();
        } else {
            d[0] = m.at("mua").as_float() * s.unitinmm;
            d[1] = m.at("mus").as_float() * s.unitinmm;
            d[2] = m.at("g").as_float();
            d[3] = m.at("n").as_float();
        }
    }
    // detectors (L808-810)
    job.detpos.resize(static_cast<size_t>(s.detnum) * 4);
    for (int i = 0; i < s.detnum; i++) {
        const Value& d = optode->at("Detector").at(static_cast<size_t>(i));
        float* o = &job.detpos[static_cast<size_t>(i) * 4];
        for (int k = 0; k < 3; k++) o[k] = d.at("Pos").at(static_cast<size_t>(k)).as_float();
        o[3] = d.at("R").as_float();
    }
    // labels: int32 + sign-bit detector flag -> uint8 + bit 7 (built by umcx_gpu_build_labels instead when the
    // domain is made on the device)
    if (io.domain_on_device) return job;
    job.labels.resize(io.domain.vol.size());
    for (size_t i = 0; i < io.domain.vol.size(); i++) {
        const int32_t v = io.domain.vol[i];
        const int32_t med = v & kMedMask;
        if (med >= s.mediumnum || med > static_cast<int32_t>(UMCX_LABEL_MASK))
            throw std::runtime_error("label " + std::to_string(med) + " has no entry in Domain.Media");
        job.labels[i] = static_cast<uint8_t>(med | ((v & kDetMask) ? UMCX_LABEL_DET : 0u));
    }
    return job;
}

}  // namespace umcx

// host-side parts of the C ABI (umcx_gpu.h): the detected-photon record width (L157) and the session seeds
// (L724-727)
extern "C" int umcx_detp_columns(const umcx_sim* s) {
    if (!s) return 0;
    return (s->savedetflag & UMCX_DET_ID) + ((s->savedetflag & UMCX_DET_PPATH) > 0) * s->mediumnum +
           (((s->savedetflag & UMCX_DET_EXITPOS) > 0) + ((s->savedetflag & UMCX_DET_EXITDIR) > 0)) * 3;
}

extern "C" int umcx_seeds_from_rngseed(int32_t rngseed, uint32_t seeds[4]) {
    if (!seeds) return UMCX_ERR_INPUT;
    // srand(seed) followed by four rand() calls of the C library (L724-727), through the reentrant interface so
    // the caller's own rand() state is left alone; rngseed <= 0 means "seed from the clock" like the reference
    unsigned seed = rngseed > 0 ? static_cast<unsigned>(rngseed) : static_cast<unsigned>(std::time(nullptr));
    struct random_data rd;
    char state[128];
    std::memset(&rd, 0, sizeof(rd));
    std::memset(state, 0, sizeof(state));
    if (initstate_r(seed, state, sizeof(state), &rd) != 0) return UMCX_ERR_INPUT;
    for (int i = 0; i < 4; i++) {
        int32_t v = 0;
        random_r(&rd, &v);
        seeds[i] = static_cast<uint32_t>(v);
    }
    return UMCX_OK;
}
