// ref_driver.cpp -- command-line driver around maleadt/tracetransform's own
// C++ sources (c++/src or openmp/src), compiled against the stand-in headers
// in oracle/shim/.  TEST INFRASTRUCTURE ONLY: it produces golden outputs of
// the reference float path and times the reference's benchmark protocol.
//
//   ttref transform <img.f32> <rows> <cols> <step> <T,..> <P,..|-> <prefix>
//       runs Transformer::getTransform's steps (c++/src/transform.cpp:28-112)
//       and writes <prefix>.{padded,sino,nos,circus,sig}.f32 and <prefix>.meta
//   ttref rotate <img.f32> <rows> <cols> <angle_deg> <out.f32>
//       rotate() about ((cols-1)/2, (rows-1)/2) (c++/src/rottest.cpp:46-49)
//   ttref resize <img.f32> <rows> <cols> <out_rows> <out_cols> <out.f32>
//       resize() (c++/src/auxiliary.cpp:198-221)
//   ttref netpbm <in.pgm|in.ppm> <prefix>
//       readnetpbm() (c++/src/auxiliary.cpp:47-99); per channel i writes
//       <prefix>.c<i>.i32 (the pixels), <prefix>.c<i>.gray.f32 (gray2mat,
//       :148-157) and <prefix>.c<i>.pgm (writepgm, :101-128); <prefix>.meta
//   ttref mat2gray <img.f32> <rows> <cols> <prefix>
//       mat2gray() (:159-178): <prefix>.i32 and writepgm of it, <prefix>.pgm
//   ttref bench <img.f32> <rows> <cols> <step> <T,..> <P,..|-> <iterations>
//       demo.cpp's benchmark mode (c++/src/demo.cpp:222-248): one warm-up and
//       <iterations> timed getTransform(..., false) calls; prints t_i=<s>
//
// Images are raw float32, column-major (Eigen order), already scaled to
// [0, 1] as gray2mat does (c++/src/auxiliary.cpp:148-157).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "auxiliary.hpp"
#include "circus.hpp"
#include "sinogram.hpp"
#include "transform.hpp"

static Eigen::MatrixXf read_image(const char *path, int rows, int cols) {
    Eigen::MatrixXf m = Eigen::MatrixXf::Zero(rows, cols);
    std::ifstream f(path, std::ios::binary);
    if (!f.good())
        throw std::runtime_error("cannot open image file");
    f.read(reinterpret_cast<char *>(m.data()),
           sizeof(float) * (size_t)rows * cols);
    if (!f)
        throw std::runtime_error("short image file");
    return m;
}

static void write_floats(const std::string &path, const float *p, size_t n) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char *>(p), sizeof(float) * n);
}

template <typename W>
static std::vector<W> parse_list(const std::string &spec) {
    std::vector<W> out;
    if (spec == "-")
        return out;
    std::stringstream ss(spec);
    std::string item;
    while (std::getline(ss, item, ',')) {
        std::istringstream in(item);
        W w;
        in >> w; // the reference's own operator>> parsers
        out.push_back(w);
    }
    return out;
}

static bool orthonormal_mode(const std::vector<PFunctionalWrapper> &pf) {
    // c++/src/demo.cpp:153-169
    size_t count = 0;
    for (size_t p = 0; p < pf.size(); p++)
        if (pf[p].functional == PFunctional::Hermite)
            count++;
    if (count == 0)
        return false;
    if (count == pf.size())
        return true;
    throw std::runtime_error("Cannot mix regular and orthonormal P-functionals");
}

static int do_transform(int argc, char **argv) {
    if (argc != 9)
        return 2;
    int rows = atoi(argv[3]), cols = atoi(argv[4]);
    unsigned step = (unsigned)atoi(argv[5]);
    std::vector<TFunctionalWrapper> tf = parse_list<TFunctionalWrapper>(argv[6]);
    std::vector<PFunctionalWrapper> pf = parse_list<PFunctionalWrapper>(argv[7]);
    std::string prefix = argv[8];
    bool ortho = orthonormal_mode(pf);

    Eigen::MatrixXf image = read_image(argv[2], rows, cols);
    // Transformer::Transformer (c++/src/transform.cpp:28-47)
    if (ortho) {
        size_t ndiag = (int)std::ceil(360.0 / step);
        size_t nsize = (int)std::ceil(ndiag / std::sqrt(2));
        image = resize(image, nsize, nsize);
    }
    image = pad(image);
    write_floats(prefix + ".padded.f32", image.data(), image.size());

    // Transformer::getTransform (c++/src/transform.cpp:49-112)
    int a_steps = (int)std::floor(360 / step);
    std::vector<Eigen::MatrixXf> sinograms = getSinograms(image, step, tf);
    std::vector<float> sino, nos, circus, sig((size_t)a_steps * tf.size() * pf.size());
    std::vector<long> centers, nos_rows;
    for (size_t t = 0; t < tf.size(); t++) {
        sino.insert(sino.end(), sinograms[t].data(),
                    sinograms[t].data() + sinograms[t].size());
        if (ortho) {
            size_t center;
            sinograms[t] = nearest_orthonormal_sinogram(sinograms[t], center);
            for (size_t p = 0; p < pf.size(); p++)
                if (pf[p].functional == PFunctional::Hermite)
                    pf[p].arguments.center = center;
            centers.push_back((long)center);
            nos_rows.push_back((long)sinograms[t].rows());
            nos.insert(nos.end(), sinograms[t].data(),
                       sinograms[t].data() + sinograms[t].size());
        }
        if (pf.size() > 0) {
            std::vector<Eigen::VectorXf> cf = getCircusFunctions(sinograms[t], pf);
            for (size_t p = 0; p < pf.size(); p++) {
                circus.insert(circus.end(), cf[p].data(), cf[p].data() + cf[p].size());
                Eigen::VectorXf z = zscore(cf[p]);
                for (int a = 0; a < a_steps; a++)
                    sig[(size_t)a + (t * pf.size() + p) * a_steps] = z[a];
            }
        }
    }
    write_floats(prefix + ".sino.f32", sino.data(), sino.size());
    write_floats(prefix + ".circus.f32", circus.data(), circus.size());
    write_floats(prefix + ".sig.f32", sig.data(), sig.size());
    if (ortho)
        write_floats(prefix + ".nos.f32", nos.data(), nos.size());
    std::ofstream meta(prefix + ".meta");
    meta << "n " << image.rows() << "\nangles " << a_steps << "\northo "
         << (ortho ? 1 : 0) << "\n";
    for (size_t t = 0; t < centers.size(); t++)
        meta << "center " << centers[t] << " " << nos_rows[t] << "\n";
    return 0;
}

static int do_rotate(int argc, char **argv) {
    if (argc != 7)
        return 2;
    int rows = atoi(argv[3]), cols = atoi(argv[4]);
    float angle = (float)atof(argv[5]);
    Eigen::MatrixXf input = read_image(argv[2], rows, cols);
    Point<float>::type origin((input.cols() - 1) / 2.0, (input.rows() - 1) / 2.0);
    Eigen::MatrixXf out = rotate(input, origin, deg2rad(angle));
    write_floats(argv[6], out.data(), out.size());
    return 0;
}

static int do_resize(int argc, char **argv) {
    if (argc != 8)
        return 2;
    int rows = atoi(argv[3]), cols = atoi(argv[4]);
    int out_rows = atoi(argv[5]), out_cols = atoi(argv[6]);
    Eigen::MatrixXf out = resize(read_image(argv[2], rows, cols), out_rows, out_cols);
    write_floats(argv[7], out.data(), out.size());
    return 0;
}

static void write_ints(const std::string &path, const Eigen::MatrixXi &m) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char *>(m.data()), sizeof(int) * (size_t)m.size());
}

static int do_netpbm(int argc, char **argv) {
    if (argc != 4)
        return 2;
    std::string prefix = argv[3];
    std::vector<Eigen::MatrixXi> components = readnetpbm(argv[2]);
    std::ofstream meta(prefix + ".meta");
    meta << "channels " << components.size() << "\n";
    for (size_t i = 0; i < components.size(); i++) {
        const std::string base = prefix + ".c" + std::to_string(i);
        meta << "shape " << components[i].rows() << " " << components[i].cols() << "\n";
        write_ints(base + ".i32", components[i]);
        Eigen::MatrixXf gray = gray2mat(components[i]);
        write_floats(base + ".gray.f32", gray.data(), gray.size());
        writepgm(base + ".pgm", components[i]);
    }
    return 0;
}

static int do_mat2gray(int argc, char **argv) {
    if (argc != 6)
        return 2;
    int rows = atoi(argv[3]), cols = atoi(argv[4]);
    std::string prefix = argv[5];
    Eigen::MatrixXi gray = mat2gray(read_image(argv[2], rows, cols));
    write_ints(prefix + ".i32", gray);
    writepgm(prefix + ".pgm", gray);
    return 0;
}

static int do_bench(int argc, char **argv) {
    if (argc != 9)
        return 2;
    int rows = atoi(argv[3]), cols = atoi(argv[4]);
    unsigned step = (unsigned)atoi(argv[5]);
    std::vector<TFunctionalWrapper> tf = parse_list<TFunctionalWrapper>(argv[6]);
    std::vector<PFunctionalWrapper> pf = parse_list<PFunctionalWrapper>(argv[7]);
    unsigned iterations = (unsigned)atoi(argv[8]);
    bool ortho = orthonormal_mode(pf);
    Transformer transformer(read_image(argv[2], rows, cols), "bench", step, ortho);
    transformer.getTransform(tf, pf, false);
    for (unsigned n = 0; n < iterations; n++) {
        auto last = std::chrono::high_resolution_clock::now();
        transformer.getTransform(tf, pf, false);
        auto current = std::chrono::high_resolution_clock::now();
        std::cout << "t_" << n + 1 << "="
                  << std::chrono::duration_cast<std::chrono::microseconds>(
                         current - last).count() / 1000000.0
                  << std::endl;
    }
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        std::cerr << "usage: ttref transform|rotate|resize|netpbm|mat2gray|bench ..." << std::endl;
        return 2;
    }
    std::string mode = argv[1];
    int rc = 2;
    try {
        if (mode == "transform")
            rc = do_transform(argc, argv);
        else if (mode == "rotate")
            rc = do_rotate(argc, argv);
        else if (mode == "bench")
            rc = do_bench(argc, argv);
        else if (mode == "resize")
            rc = do_resize(argc, argv);
        else if (mode == "netpbm")
            rc = do_netpbm(argc, argv);
        else if (mode == "mat2gray")
            rc = do_mat2gray(argc, argv);
    } catch (const std::exception &e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 1;
    }
    if (rc == 2)
        std::cerr << "bad arguments" << std::endl;
    return rc;
}
