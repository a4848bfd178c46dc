// test_api.cpp -- C++ tests of the drop-in API (run / TSFOutput / paramList),
// written after the reference's GTest suites (tests/parameterTests.cpp,
// tests/TSFOutputTests.cpp, tests/tubeSegmentationTests.cpp) with a minimal
// assertion layer (GTest is not available).
//
//   test_api cpu                 parameter, TSFOutput and I/O tests (no GPU)
//   test_api bench <file.mhd> <repeats> [--name value ...]
//                                run() timed end to end (one JSON line)
//   test_api run <file.mhd> <out_dir> [--name value ...]
//                                run() on a volume; writes tdf.raw (float),
//                                centerline.raw (int8), segmentation.raw
//                                (int8, when there is one), vertices.txt,
//                                size.txt and shift.txt
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "tsf/tube-segmentation.hpp"

static int g_failures = 0, g_checks = 0;

#define EXPECT_TRUE(c)                                                                   \
    do {                                                                                 \
        g_checks++;                                                                      \
        if (!(c)) {                                                                      \
            g_failures++;                                                                \
            std::cerr << __FILE__ << ":" << __LINE__ << ": expected " #c << std::endl;   \
        }                                                                                \
    } while (0)
#define EXPECT_FALSE(c) EXPECT_TRUE(!(c))
#define EXPECT_EQ(a, b) EXPECT_TRUE((a) == (b))
#define EXPECT_THROW(stmt, ex)                                                           \
    do {                                                                                 \
        bool thrown = false;                                                             \
        try { stmt; } catch (const ex &) { thrown = true; } catch (...) {}               \
        EXPECT_TRUE(thrown && "throws " #ex);                                            \
    } while (0)
#define EXPECT_NO_THROW(stmt)                                                            \
    do {                                                                                 \
        bool thrown = false;                                                             \
        try { stmt; } catch (...) { thrown = true; }                                     \
        EXPECT_TRUE(!thrown && "does not throw");                                        \
    } while (0)

// ---- parameterTests.cpp ----------------------------------------------------
static void parameter_tests() {
    paramList parameters = initParameters(PARAMETERS_DIR);
    EXPECT_FALSE(getParamBool(parameters, "display"));
    EXPECT_EQ(std::string("gpu"), getParamStr(parameters, "device"));
    EXPECT_EQ(0.05f, getParam(parameters, "gvf-mu"));
    EXPECT_EQ(std::string("Display results"), parameters.bools["display"].getDescription());
    EXPECT_EQ(std::string("Which type of processor to use"), parameters.strings["device"].getDescription());
    EXPECT_EQ(std::string("Mu regularization constant of GVF"), parameters.numerics["gvf-mu"].getDescription());

    setParameter(parameters, "display", "true");
    EXPECT_TRUE(getParamBool(parameters, "display"));
    setParameter(parameters, "cropping", "lung");
    EXPECT_EQ(std::string("lung"), getParamStr(parameters, "cropping"));
    setParameter(parameters, "tdf-high", "0.9");
    EXPECT_EQ(0.9f, getParam(parameters, "tdf-high"));
    EXPECT_THROW(setParameter(parameters, "no-such-parameter", "1"), SIPL::SIPLException);
    EXPECT_THROW(setParameter(parameters, "mode", "grey"), SIPL::SIPLException);
    EXPECT_THROW(getParam(parameters, "mode"), SIPL::SIPLException);

    NumericParameter p;
    EXPECT_NO_THROW(p = NumericParameter(0.2f, 0.1f, 1.0f, 0.1f, "asd", "asd"));
    EXPECT_THROW(p.set(0.05f), SIPL::SIPLException);
    EXPECT_THROW(p.set(1.2f), SIPL::SIPLException);
    EXPECT_NO_THROW(p.set(0.4f));

    std::vector<std::string> possibilities = {"test", "moretest", "evenmoretest"};
    StringParameter sp;
    EXPECT_NO_THROW(sp = StringParameter("test", possibilities, "asd", "asd"));
    EXPECT_THROW(sp.set("abc"), SIPL::SIPLException);

    BoolParameter b(true, "test description", "asd");
    EXPECT_EQ(std::string("test description"), b.getDescription());
    EXPECT_EQ(std::string("asd"), b.getGroup());
    paramList q = initParameters(PARAMETERS_DIR);
    EXPECT_EQ(std::string("Extract black or white tubular structures"), q.strings["mode"].getDescription());
    EXPECT_EQ(std::string("Minimum radius of tubular structures"), q.numerics["radius-min"].getDescription());
    EXPECT_EQ(std::string("advanced"), q.bools["display"].getGroup());
    EXPECT_EQ(std::string("general"), q.strings["mode"].getGroup());
    EXPECT_EQ(std::string("tube-detection-filter"), q.numerics["radius-min"].getGroup());

    // presets (tubeSegmentationTests.cpp:15-22)
    setParameter(q, "parameters", "Synthetic-Vascusynth");
    setParameter(q, "centerline-method", "gpu");
    loadParameterPreset(q, PARAMETERS_DIR);
    EXPECT_EQ(0.35f, getParam(q, "tdf-high"));
    EXPECT_EQ(3.0f, getParam(q, "cube-size"));
    EXPECT_EQ(4.0f, getParam(q, "radius-max"));
    EXPECT_EQ(std::string("75"), getParamStr(q, "maximum"));
    paramList r = initParameters(PARAMETERS_DIR);
    setParameter(r, "parameters", "No-Such-Preset");
    EXPECT_THROW(loadParameterPreset(r, PARAMETERS_DIR), SIPL::IOException);
    EXPECT_THROW(initParameters("/nonexistent-parameter-dir"), SIPL::IOException);

    // command line (parameters.cpp:227-270)
    const char *argv[] = {"tsf", "vol.mhd", "--parameters", "Synthetic-Vascusynth", "--gvf-iterations", "100",
                          "--tdf-only"};
    paramList c = getParameters(7, const_cast<char **>(argv));
    EXPECT_EQ(100.0f, getParam(c, "gvf-iterations"));
    EXPECT_TRUE(getParamBool(c, "tdf-only"));
    EXPECT_EQ(0.1f, getParam(c, "fmax"));
}

// ---- TSFOutputTests.cpp ------------------------------------------------------
static void output_tests() {
    {
        TSFOutput output(oul::DeviceCriteria(), new SIPL::int3);
        EXPECT_FALSE(output.hasSegmentation());
        EXPECT_FALSE(output.hasCenterlineVoxels());
        EXPECT_FALSE(output.hasTDF());
        EXPECT_THROW(output.getTDF(), SIPL::SIPLException);
    }
    {
        TSFOutput output(oul::DeviceCriteria(), new SIPL::int3);
        output.setTDF(new float[1]);
        EXPECT_TRUE(output.hasTDF());
        EXPECT_FALSE(output.hasSegmentation());
        output.setSegmentation(new char[1]);
        EXPECT_TRUE(output.hasSegmentation());
        EXPECT_FALSE(output.hasCenterlineVoxels());
        output.setCenterlineVoxels(new char[1]);
        EXPECT_TRUE(output.hasCenterlineVoxels());
    }
    {
        TSFOutput output(oul::DeviceCriteria(), new SIPL::int3);
        float *TDF = new float[3]{0.5f, 1.0f, 0.0f};
        output.setTDF(TDF);
        EXPECT_EQ(0.5f, output.getTDF()[0]);
        EXPECT_EQ(1.0f, output.getTDF()[1]);
        EXPECT_EQ(0.0f, output.getTDF()[2]);
        char *data = new char[3]{1, 2, 100};
        output.setSegmentation(data);
        EXPECT_EQ(100, output.getSegmentation()[2]);
        char *data2 = new char[3]{10, 20, 10};
        output.setCenterlineVoxels(data2);
        EXPECT_EQ(20, output.getCenterlineVoxels()[1]);
    }
    {
        TSFOutput output(oul::DeviceCriteria(), new SIPL::int3(100, 20, 1));
        EXPECT_EQ(100, output.getSize()->x);
        EXPECT_EQ(20, output.getSize()->y);
        EXPECT_EQ(1, output.getSize()->z);
    }
    {
        TSFOutput output(oul::DeviceCriteria(), new SIPL::int3);
        output.setShiftVector(SIPL::int3(3, 10, 2));
        EXPECT_EQ(3, output.getShiftVector().x);
        EXPECT_EQ(10, output.getShiftVector().y);
        EXPECT_EQ(2, output.getShiftVector().z);
    }
}

// ---- tubeSegmentationTests.cpp:4-7 and option checks (no GPU needed) ----------
static void io_tests() {
    paramList parameters = initParameters(PARAMETERS_DIR);
    EXPECT_THROW(run("somefilethatdoesntexist.mhd", parameters, KERNELS_DIR), SIPL::IOException);
    EXPECT_THROW(runSegmentation("somefilethatdoesntexist.mhd", parameters, KERNELS_DIR), SIPL::IOException);
    paramList p2 = initParameters(PARAMETERS_DIR);
    setParameter(p2, "centerline-method", "ridge");
    EXPECT_THROW(run("x.mhd", p2, KERNELS_DIR), SIPL::SIPLException);
    paramList p3 = initParameters(PARAMETERS_DIR);
    setParameter(p3, "device", "cpu");
    EXPECT_THROW(run("x.mhd", p3, KERNELS_DIR), SIPL::SIPLException);
    // a .raw file shorter than DimSize x the element size: IOException before any device call
    // (the read splits the file over threads; a short slice fails the whole read)
    const std::string name = "tsf_api_truncated_" + std::to_string((long long)std::chrono::steady_clock::now()
                                                                        .time_since_epoch()
                                                                        .count());
    const std::string base = "/tmp/" + name;
    {
        std::ofstream(base + ".mhd") << "ObjectType = Image\nNDims = 3\nDimSize = 256 256 160\n"
                                        "ElementType = MET_FLOAT\nElementDataFile = " << name << ".raw\n";
        std::vector<float> part((size_t)256 * 256 * 159, 0.5f);   // one plane short of 40 MB
        FILE *f = std::fopen((base + ".raw").c_str(), "wb");
        std::fwrite(part.data(), sizeof(float), part.size(), f);
        std::fclose(f);
    }
    paramList p4 = initParameters(PARAMETERS_DIR);
    EXPECT_THROW(run(base + ".mhd", p4, KERNELS_DIR), SIPL::IOException);
    std::remove((base + ".mhd").c_str());
    std::remove((base + ".raw").c_str());
}

static int run_mode(int argc, char **argv) {
    // argv: test_api run <file.mhd> <out_dir> [--name value ...]
    std::vector<char *> args;
    args.push_back(argv[0]);
    args.push_back(argv[2]);
    for (int i = 4; i < argc; i++) args.push_back(argv[i]);
    paramList parameters = getParameters((int)args.size(), args.data());
    const std::string out = argv[3];
    TSFOutput *o = nullptr;
    try {
        o = run(argv[2], parameters, KERNELS_DIR);
    } catch (const SIPL::SIPLException &e) {
        std::cerr << "SIPLException: " << e.what() << std::endl;
        return 3;
    }
    const SIPL::int3 s = *o->getSize();
    const size_t n = (size_t)s.x * s.y * s.z;
    std::ofstream(out + "/size.txt") << s.x << " " << s.y << " " << s.z << "\n";
    const SIPL::int3 sh = o->getShiftVector();
    std::ofstream(out + "/shift.txt") << sh.x << " " << sh.y << " " << sh.z << "\n";
    {
        FILE *f = std::fopen((out + "/tdf.raw").c_str(), "wb");
        std::fwrite(o->getTDF(), sizeof(float), n, f);
        std::fclose(f);
    }
    if (o->hasCenterlineVoxels()) {
        FILE *f = std::fopen((out + "/centerline.raw").c_str(), "wb");
        std::fwrite(o->getCenterlineVoxels(), 1, n, f);
        std::fclose(f);
    }
    if (o->hasSegmentation()) {
        FILE *f = std::fopen((out + "/segmentation.raw").c_str(), "wb");
        std::fwrite(o->getSegmentation(), 1, n, f);
        std::fclose(f);
    }
    std::ofstream vt(out + "/vertices.txt");
    for (const auto &v : o->getCenterpoints()) vt << v.x << " " << v.y << " " << v.z << "\n";
    delete o;
    return 0;
}

// argv: test_api bench <file.mhd> <repeats> [--name value ...]: run() once
// to warm up, then `repeats` times, each timed end to end on the host clock
// (the file read, the uploads, the whole pipeline and the copies of the TDF,
// centerline and segmentation the getters make) and printed as one JSON line.
static int bench_mode(int argc, char **argv) {
    std::vector<char *> args;
    args.push_back(argv[0]);
    args.push_back(argv[2]);
    for (int i = 4; i < argc; i++) args.push_back(argv[i]);
    const int repeats = std::atoi(argv[3]);
    std::vector<double> ms, run_ms, get_ms;
    size_t vertices = 0, segmented = 0;
    for (int k = -1; k < repeats; k++) {
        paramList parameters = getParameters((int)args.size(), args.data());
        const auto t0 = std::chrono::steady_clock::now();
        TSFOutput *o = nullptr;
        try {
            o = run(argv[2], parameters, KERNELS_DIR);
        } catch (const SIPL::SIPLException &e) {
            std::cerr << "SIPLException: " << e.what() << std::endl;
            return 3;
        }
        const auto tr = std::chrono::steady_clock::now();
        const SIPL::int3 s = *o->getSize();
        const size_t n = (size_t)s.x * s.y * s.z;
        const float *tdf = o->getTDF();
        const char *cl = o->hasCenterlineVoxels() ? o->getCenterlineVoxels() : nullptr;
        const char *seg = o->hasSegmentation() ? o->getSegmentation() : nullptr;
        const auto t1 = std::chrono::steady_clock::now();
        if (k >= 0) {
            ms.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
            run_ms.push_back(std::chrono::duration<double, std::milli>(tr - t0).count());
            get_ms.push_back(std::chrono::duration<double, std::milli>(t1 - tr).count());
        }
        vertices = o->getCenterpoints().size();
        segmented = 0;
        if (seg)
            for (size_t i = 0; i < n; i++) segmented += seg[i] != 0;
        (void)tdf;
        (void)cl;
        delete o;
    }
    auto list = [](const char *key, const std::vector<double> &v) {
        std::cout << "\"" << key << "\": [";
        for (size_t i = 0; i < v.size(); i++) std::cout << (i ? ", " : "") << v[i];
        std::cout << "], ";
    };
    std::cout << "{";
    list("run_ms", ms);
    list("run_call_ms", run_ms);
    list("getters_ms", get_ms);
    std::cout << "\"vertices\": " << vertices << ", \"segmented_voxels\": " << segmented << "}" << std::endl;
    return 0;
}

int main(int argc, char **argv) {
    const std::string mode = argc > 1 ? argv[1] : "cpu";
    if (mode == "run" && argc >= 4) return run_mode(argc, argv);
    if (mode == "bench" && argc >= 4) return bench_mode(argc, argv);
    parameter_tests();
    output_tests();
    io_tests();
    std::cout << g_checks << " checks, " << g_failures << " failures" << std::endl;
    return g_failures ? 1 : 0;
}
