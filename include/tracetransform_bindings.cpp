// tracetransform_bindings.cpp -- the reference-side bindings of the engine.
//
// A maintainer of maleadt/tracetransform's C++ port links it against
// libtt_gb300.so by replacing the bodies of the functions below in the
// reference (each keeps the reference's own declaration, from its headers
// c++/src/sinogram.hpp, circus.hpp and auxiliary.hpp):
//
//   getSinograms                  c++/src/sinogram.cpp:67-178
//   getCircusFunctions            c++/src/circus.cpp:104-177
//   nearest_orthonormal_sinogram  c++/src/circus.cpp:68-102
//   zscore                        c++/src/auxiliary.cpp:305-318
//   resize                        c++/src/auxiliary.cpp:198-221
//
// and, optionally, Transformer::getTransform (c++/src/transform.cpp:49-112)
// with one tt_transform call per image component (transform_image below) or
// the reference demo's loop over its inputs (c++/src/demo.cpp:179-254) with
// one tt_transform_batch call (transform_batch below).
//
// The reference's matrices are Eigen column-major, the ABI's layout, so the
// data() pointers go straight through.  Compiled against the reference's
// headers by oracle/check_integration.py (tests/test_integration_bindings.py)
// with missing declarations as errors, so every signature is the reference's.
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <vector>

#include <boost/program_options.hpp> // validation_error, as the reference throws it

#include "auxiliary.hpp"
#include "circus.hpp"
#include "sinogram.hpp"
#include "tracetransform.h"

static void tt_check(tt_status st) {
    if (st == TT_ERR_INVALID_ARG)
        throw boost::program_options::validation_error(
            boost::program_options::validation_error::invalid_option_value);
    if (st != TT_OK)
        throw std::runtime_error(tt_last_error());
}

std::vector<Eigen::MatrixXf>
getSinograms(const Eigen::MatrixXf &input, unsigned int angle_stepsize,
             const std::vector<TFunctionalWrapper> &tfunctionals) {
    const int a_steps = (int)std::floor(360 / angle_stepsize);
    std::vector<int32_t> ids;
    for (const auto &t : tfunctionals)
        ids.push_back((int32_t)t.functional); // enum order == TT_T_RADON..TT_T7
    std::vector<float> out(ids.size() * input.rows() * a_steps);
    tt_check(tt_sinograms(nullptr, input.data(), input.rows(), input.cols(),
                          angle_stepsize, ids.data(), (int)ids.size(), out.data()));
    std::vector<Eigen::MatrixXf> result;
    for (size_t t = 0; t < ids.size(); t++)
        result.push_back(Eigen::Map<Eigen::MatrixXf>(
            out.data() + t * input.rows() * a_steps, input.rows(), a_steps));
    return result;
}

static std::vector<tt_pfunctional> to_tt(const std::vector<PFunctionalWrapper> &pfunctionals) {
    std::vector<tt_pfunctional> pf;
    for (const auto &p : pfunctionals) {
        tt_pfunctional f;
        f.kind = p.functional == PFunctional::Hermite ? TT_P_HERMITE
                 : p.functional == PFunctional::P1    ? TT_P1
                 : p.functional == PFunctional::P2    ? TT_P2 : TT_P3;
        f.order = p.arguments.order ? (int32_t)*p.arguments.order : -1;
        f.center = p.arguments.center ? (int32_t)*p.arguments.center : -1;
        pf.push_back(f);
    }
    return pf;
}

std::vector<Eigen::VectorXf>
getCircusFunctions(const Eigen::MatrixXf &input,
                   const std::vector<PFunctionalWrapper> &pfunctionals) {
    const std::vector<tt_pfunctional> pf = to_tt(pfunctionals);
    std::vector<float> out(pf.size() * input.cols());
    tt_check(tt_circus(nullptr, input.data(), input.rows(), input.cols(),
                       pf.data(), (int)pf.size(), out.data()));
    std::vector<Eigen::VectorXf> result;
    for (size_t p = 0; p < pf.size(); p++)
        result.push_back(Eigen::Map<Eigen::VectorXf>(out.data() + p * input.cols(),
                                                     input.cols()));
    return result;
}

Eigen::MatrixXf nearest_orthonormal_sinogram(const Eigen::MatrixXf &input,
                                             size_t &new_center) {
    std::vector<float> out(2 * input.rows() * input.cols());
    int32_t m = 0, c = 0;
    tt_check(tt_nos(nullptr, input.data(), input.rows(), input.cols(), out.data(), &m, &c));
    new_center = (size_t)c;
    return Eigen::Map<Eigen::MatrixXf>(out.data(), m, input.cols());
}

Eigen::VectorXf zscore(const Eigen::VectorXf &input) {
    Eigen::VectorXf out(input.size());
    if (input.size())
        tt_check(tt_zscore(nullptr, input.data(), 1, input.size(), out.data()));
    return out;
}

Eigen::MatrixXf resize(const Eigen::MatrixXf &input, const size_t rows, const size_t cols) {
    Eigen::MatrixXf out(rows, cols);
    tt_check(tt_resize(nullptr, input.data(), input.rows(), input.cols(), rows, cols,
                       out.data()));
    return out;
}

// The body of Transformer::getTransform for one image component: the
// orthonormal stretch, padding, sinograms, nearest orthonormal sinogram,
// circus functions and z-scores in one call.  Returns the A x (nT nP)
// signature matrix the reference writes to <basename>.csv.
[[maybe_unused]] static Eigen::MatrixXf
transform_image(const Eigen::MatrixXf &image, unsigned angle_stepsize,
                const std::vector<TFunctionalWrapper> &tfunctionals,
                const std::vector<PFunctionalWrapper> &pfunctionals) {
    std::vector<int32_t> ids;
    for (const auto &t : tfunctionals)
        ids.push_back((int32_t)t.functional);
    const std::vector<tt_pfunctional> pf = to_tt(pfunctionals);
    int A = 0;
    tt_check(tt_angles_from_step(angle_stepsize, nullptr, 0, &A));
    const int nT = (int)ids.size(), nP = (int)pf.size();
    std::vector<float> circus(nT * nP * A), signatures(nT * nP * A);
    tt_check(tt_transform(nullptr, image.data(), image.rows(), image.cols(),
                          angle_stepsize, ids.data(), nT, pf.data(), nP,
                          circus.data(), signatures.data()));
    return Eigen::Map<Eigen::MatrixXf>(signatures.data(), A, nT * nP);
}

// The demo's loop over its inputs as one batched call: images column-major
// back to back, offsets[i] the first element of image i; circus and
// signatures receive each image's nT x nP x A_i block in turn.
[[maybe_unused]] static void
transform_batch(const float *images, const int64_t *offsets, const int32_t *rows,
                const int32_t *cols, const int32_t *angle_steps, int n_images,
                const int32_t *ids, int nT, const tt_pfunctional *pf, int nP, float *circus,
                float *signatures) {
    tt_check(tt_transform_batch(nullptr, images, offsets, rows, cols, angle_steps, n_images,
                                ids, nT, pf, nP, circus, signatures));
}
