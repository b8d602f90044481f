/* Header-only C++ facade over the C ABI (tw_dic.h): the reference engine's
 * six DIC class shapes and method names (TW/TW_Engine/TW_paDIC_FFTCC2D.h,
 * TW_paDIC_FFTCC2D_CPU.h, TW_paDIC_cuFFTCC2D.h, TW_paDIC_ICGN2D.h,
 * TW_paDIC_ICGN2D_CPU.h, TW_paDIC_cuICGN2D.h) in namespace TW::paDIC, so that
 * a caller of those classes recompiles against this header and links
 * libtwdic.so.
 *
 * Differences a caller sees:
 *   - images are a small view {data, width, height, step} (ImageView)
 *     instead of cv::Mat; with OpenCV included first, a cv::Mat converts to
 *     it implicitly;
 *   - errors throw std::logic_error (constructors, as the reference) or
 *     std::runtime_error (methods) with the library's message, where the
 *     reference calls exit() from checkCudaErrors;
 *   - the "CPU" classes compute on the GPU with the reference CPU path's
 *     semantics (first-maximum FFT-CC peak, integer first IC-GN pass,
 *     OutofROI / dark / singular flags, Cholesky solve); paDICThreadFlag is
 *     accepted and ignored;
 *   - cuICGN2D borrows nothing it frees: images and POIs are copied into the
 *     handle, so a caller that shares device arrays with cuFFTCC2D does not
 *     double-free them (TW_paDIC_cuICGN2D.cu:719-729 frees borrowed arrays);
 *   - SetTarImg sets the target (the reference's cuICGN2D::SetTarImg writes
 *     into the reference buffer, TW_paDIC_cuICGN2D.cu:805);
 * real_t is float (the reference's default build). */
#ifndef TW_DIC_HPP
#define TW_DIC_HPP

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "tw_dic.h"

namespace TW {

using real_t = float;
using int_t = int;

namespace paDIC {

enum class ICGN2DFlag { Success, DarkSubset, SingularHessian, SingularWarp, OutofROI };
enum class paDICThreadFlag { Single, Multicore };
enum class ICGN2DInterpolationFLag { Bicubic, BicubicSpline };

/* 8-bit single-channel image: `step` bytes between rows; `on_device` marks a
 * device pointer. */
struct ImageView {
    const unsigned char* data = nullptr;
    int cols = 0;
    int rows = 0;
    int step = 0;
    bool on_device = false;
    ImageView() = default;
    ImageView(const unsigned char* d, int width, int height, int step_bytes = 0, bool device = false)
        : data(d), cols(width), rows(height), step(step_bytes ? step_bytes : width), on_device(device) {}
#ifdef CV_VERSION_MAJOR
    ImageView(const cv::Mat& m) : data(m.data), cols(m.cols), rows(m.rows), step((int)m.step[0]) {}
#endif
};

namespace detail {

inline std::string last_error() {
    const char* m = twdic_last_error();
    return m ? std::string(m) : std::string();
}
inline void check(int rc, const char* what) {
    if (rc != TWDIC_OK) throw std::runtime_error(std::string(what) + ": " + last_error());
}
inline void check_ctor(int rc, const char* what) {
    if (rc != TWDIC_OK) throw std::logic_error(std::string(what) + ": " + last_error());
}
inline int mem_of(const ImageView& im) { return im.on_device ? TWDIC_MEM_DEVICE : TWDIC_MEM_HOST; }

/* Contiguous 2-D / 3-D host arrays with row pointers (the reference's
 * hcreateptr layout): a[y][x] with a[0] the whole block. */
template <typename T>
T** create2d(int ny, int nx) {
    T** rows = new T*[ny];
    T* block = new T[(size_t)ny * nx]();
    for (int y = 0; y < ny; ++y) rows[y] = block + (size_t)y * nx;
    return rows;
}
template <typename T>
void destroy2d(T**& a) {
    if (!a) return;
    delete[] a[0];
    delete[] a;
    a = nullptr;
}
template <typename T>
T*** create3d(int ny, int nx, int nz) {
    T*** planes = new T**[ny];
    T** rows = new T*[(size_t)ny * nx];
    T* block = new T[(size_t)ny * nx * nz]();
    for (int y = 0; y < ny; ++y) {
        planes[y] = rows + (size_t)y * nx;
        for (int x = 0; x < nx; ++x) planes[y][x] = block + ((size_t)y * nx + x) * nz;
    }
    return planes;
}
template <typename T>
void destroy3d(T***& a) {
    if (!a) return;
    delete[] a[0][0];
    delete[] a[0];
    delete[] a;
    a = nullptr;
}

}  // namespace detail

/* ------------------------------------------------------------- Fftcc2D -- */
class Fftcc2D {
public:
    Fftcc2D(const int_t iImgWidth, const int_t iImgHeight, const int_t iStartX, const int_t iStartY,
            const int_t iROIWidth, const int_t iROIHeight, const int_t iSubsetX, const int_t iSubsetY,
            const int_t iGridSpaceX, const int_t iGridSpaceY, const int_t iMarginX, const int_t iMarginY) {
        std::memset(&m_prm, 0, sizeof(m_prm));
        m_prm.img_width = iImgWidth;
        m_prm.img_height = iImgHeight;
        m_prm.start_x = iStartX;
        m_prm.start_y = iStartY;
        m_prm.roi_width = iROIWidth;
        m_prm.roi_height = iROIHeight;
        m_prm.subset_x = iSubsetX;
        m_prm.subset_y = iSubsetY;
        m_prm.grid_space_x = iGridSpaceX;
        m_prm.grid_space_y = iGridSpaceY;
        m_prm.margin_x = iMarginX;
        m_prm.margin_y = iMarginY;
        m_prm.max_iterations = 20;
        m_prm.delta_p = 0.001f;
        m_prm.path = TWDIC_PATH_FAST;
        detail::check_ctor(twdic_fftcc_create(&m_prm, &m_h), "Fftcc2D");
        int32_t nx = 0, ny = 0;
        detail::check_ctor(twdic_fftcc_num_pois(m_h, &nx, &ny), "Fftcc2D");
        m_iNumPOIX = nx;
        m_iNumPOIY = ny;
    }
    virtual ~Fftcc2D() {
        if (m_h) twdic_fftcc_destroy(m_h);
    }
    Fftcc2D(const Fftcc2D&) = delete;
    Fftcc2D& operator=(const Fftcc2D&) = delete;

    virtual void ResetRefImg(const ImageView& refImg) = 0;
    virtual void SetTarImg(const ImageView& tarImg) = 0;

    int_t GetNumPOIsX() const { return m_iNumPOIX; }
    int_t GetNumPOIsY() const { return m_iNumPOIY; }
    int_t GetNumPOIs() const { return m_iNumPOIX * m_iNumPOIY; }
    int_t GetROISize() const { return m_prm.roi_width * m_prm.roi_height; }
    int_t GetImgWidth() const { return m_prm.img_width; }
    int_t GetImgHeight() const { return m_prm.img_height; }
    int_t GetStartX() const { return m_prm.start_x; }
    int_t GetStartY() const { return m_prm.start_y; }
    int_t GetROIWidth() const { return m_prm.roi_width; }
    int_t GetROIHeight() const { return m_prm.roi_height; }
    int_t GetSubsetX() const { return m_prm.subset_x; }
    int_t GetSubsetY() const { return m_prm.subset_y; }
    int_t GetGridSpaceX() const { return m_prm.grid_space_x; }
    int_t GetGridSpaceY() const { return m_prm.grid_space_y; }
    int_t GetMarginX() const { return m_prm.margin_x; }
    int_t GetMarginY() const { return m_prm.margin_y; }

    /* POI (y, x) pairs in row-major POI order. */
    std::vector<int32_t> POIPositions() const {
        std::vector<int32_t> p(2 * (size_t)GetNumPOIs());
        detail::check(twdic_fftcc_poi_positions(m_h, p.data(), TWDIC_MEM_HOST), "POIPositions");
        return p;
    }

protected:
    void reset_ref(const ImageView& im) {
        detail::check(twdic_fftcc_reset_ref(m_h, im.data, im.step, detail::mem_of(im)), "ResetRefImg");
    }
    void set_tar(const ImageView& im) {
        detail::check(twdic_fftcc_set_tar(m_h, im.data, im.step, detail::mem_of(im)), "SetTarImg");
    }
    void compute(real_t* u, real_t* v, real_t* z, int mem) {
        detail::check(twdic_fftcc_compute(m_h, u, v, z, nullptr, mem), "ComputeFFTCC");
    }
    twdic_params m_prm;
    twdic_fftcc* m_h = nullptr;
    int_t m_iNumPOIX = 0, m_iNumPOIY = 0;
};

/* --------------------------------------------------------- Fftcc2D_CPU -- */
class Fftcc2D_CPU : public Fftcc2D {
public:
    Fftcc2D_CPU(const int_t iImgWidth, const int_t iImgHeight, const int_t iStartX, const int_t iStartY,
                const int_t iROIWidth, const int_t iROIHeight, const int_t iSubsetX, const int_t iSubsetY,
                const int_t iGridSpaceX, const int_t iGridSpaceY, const int_t iMarginX, const int_t iMarginY,
                paDICThreadFlag /*tFlag*/)
        : Fftcc2D(iImgWidth, iImgHeight, iStartX, iStartY, iROIWidth, iROIHeight, iSubsetX, iSubsetY, iGridSpaceX,
                  iGridSpaceY, iMarginX, iMarginY) {}

    void ResetRefImg(const ImageView& refImg) override { reset_ref(refImg); }
    void SetTarImg(const ImageView& tarImg) override { set_tar(tarImg); }

    /* Allocates POI[NY][NX][2] = (y, x) and U, V, ZNCC[NY][NX]. */
    void InitializeFFTCC(const ImageView& refImg, int_t***& iPOIXY, real_t**& fU, real_t**& fV, real_t**& fZNCC) {
        reset_ref(refImg);
        iPOIXY = detail::create3d<int_t>(m_iNumPOIY, m_iNumPOIX, 2);
        fU = detail::create2d<real_t>(m_iNumPOIY, m_iNumPOIX);
        fV = detail::create2d<real_t>(m_iNumPOIY, m_iNumPOIX);
        fZNCC = detail::create2d<real_t>(m_iNumPOIY, m_iNumPOIX);
        const std::vector<int32_t> p = POIPositions();
        std::memcpy(iPOIXY[0][0], p.data(), p.size() * sizeof(int32_t));
    }
    void Algorithm_FFTCC(const ImageView& tarImg, int_t*** const& /*iPOIXY*/, real_t**& fU, real_t**& fV,
                         real_t**& fZNCC) {
        set_tar(tarImg);
        compute(fU[0], fV[0], fZNCC[0], TWDIC_MEM_HOST);
    }
    void FinalizeFFTCC(int_t***& iPOIXY, real_t**& fU, real_t**& fV, real_t**& fZNCC) {
        detail::destroy3d(iPOIXY);
        detail::destroy2d(fU);
        detail::destroy2d(fV);
        detail::destroy2d(fZNCC);
    }
};

/* ----------------------------------------------------------- cuFFTCC2D -- */
class cuFFTCC2D : public Fftcc2D {
public:
    /* whole-image parameter order (TW_paDIC_cuFFTCC2D.h:52-57) */
    cuFFTCC2D(const int_t iImgWidth, const int_t iImgHeight, const int_t iROIWidth, const int_t iROIHeight,
              const int_t iStartX, const int_t iStartY, const int_t iSubsetX, const int_t iSubsetY,
              const int_t iGridSpaceX, const int_t iGridSpaceY, const int_t iMarginX, const int_t iMarginY)
        : Fftcc2D(iImgWidth, iImgHeight, iStartX, iStartY, iROIWidth, iROIHeight, iSubsetX, iSubsetY, iGridSpaceX,
                  iGridSpaceY, iMarginX, iMarginY) {}

    void ResetRefImg(const ImageView& refImg) override { reset_ref(refImg); }
    void SetTarImg(const ImageView& tarImg) override { set_tar(tarImg); }

    /* Host outputs U, V, ZNCC[NY][NX], allocated here. */
    virtual void InitializeFFTCC(real_t**& fU, real_t**& fV, real_t**& fZNCC, const ImageView& refImg) {
        reset_ref(refImg);
        fU = detail::create2d<real_t>(m_iNumPOIY, m_iNumPOIX);
        fV = detail::create2d<real_t>(m_iNumPOIY, m_iNumPOIX);
        fZNCC = detail::create2d<real_t>(m_iNumPOIY, m_iNumPOIX);
    }
    virtual void ComputeFFTCC(real_t**& fU, real_t**& fV, real_t**& fZNCC, const ImageView& tarImg) {
        set_tar(tarImg);
        compute(fU[0], fV[0], fZNCC[0], TWDIC_MEM_HOST);
    }
    virtual void DestroyFFTCC(real_t**& fU, real_t**& fV, real_t**& fZNCC) {
        detail::destroy2d(fU);
        detail::destroy2d(fV);
        detail::destroy2d(fZNCC);
    }
    /* Device outputs (cudaMalloc'd here, num_pois floats each). */
    virtual void cuInitializeFFTCC(real_t*& f_d_U, real_t*& f_d_V, real_t*& f_d_ZNCC, const ImageView& refImg) {
        reset_ref(refImg);
        const size_t b = sizeof(real_t) * (size_t)GetNumPOIs();
        if (cudaMalloc(&f_d_U, b) != cudaSuccess || cudaMalloc(&f_d_V, b) != cudaSuccess ||
            cudaMalloc(&f_d_ZNCC, b) != cudaSuccess)
            throw std::runtime_error("cuInitializeFFTCC: cudaMalloc failed");
    }
    virtual void cuComputeFFTCC(real_t*& f_d_U, real_t*& f_d_V, real_t*& f_d_ZNCC, const ImageView& tarImg) {
        set_tar(tarImg);
        compute(f_d_U, f_d_V, f_d_ZNCC, TWDIC_MEM_DEVICE);
    }
    virtual void cuDestroyFFTCC(real_t*& f_d_U, real_t*& f_d_V, real_t*& f_d_ZNCC) {
        cudaFree(f_d_U);
        cudaFree(f_d_V);
        cudaFree(f_d_ZNCC);
        f_d_U = f_d_V = f_d_ZNCC = nullptr;
    }
};

/* -------------------------------------------------------------- ICGN2D -- */
class ICGN2D {
public:
    ICGN2D(int_t iImgWidth, int_t iImgHeight, int_t iStartX, int_t iStartY, int_t iROIWidth, int_t iROIHeight,
           int_t iSubsetX, int_t iSubsetY, int_t iNumberX, int_t iNumberY, int_t iNumIterations, real_t fDeltaP) {
        std::memset(&m_prm, 0, sizeof(m_prm));
        m_prm.img_width = iImgWidth;
        m_prm.img_height = iImgHeight;
        m_prm.start_x = iStartX;
        m_prm.start_y = iStartY;
        m_prm.roi_width = iROIWidth;
        m_prm.roi_height = iROIHeight;
        m_prm.subset_x = iSubsetX;
        m_prm.subset_y = iSubsetY;
        m_prm.grid_space_x = 1;
        m_prm.grid_space_y = 1;
        m_prm.max_iterations = iNumIterations;
        m_prm.delta_p = fDeltaP;
        m_prm.path = TWDIC_PATH_FAST;
        m_iPOINumber = iNumberX * iNumberY;
        detail::check_ctor(twdic_icgn_create(&m_prm, iNumberX, iNumberY, &m_h), "ICGN2D");
    }
    virtual ~ICGN2D() {
        if (m_h) twdic_icgn_destroy(m_h);
    }
    ICGN2D(const ICGN2D&) = delete;
    ICGN2D& operator=(const ICGN2D&) = delete;

    virtual void ResetRefImg(const ImageView& refImg) = 0;
    virtual void SetTarImg(const ImageView& tarImg) = 0;
    int_t GetNumPOIs() const { return m_iPOINumber; }

    /* Per-POI flags of the last compute call (ICGN2DFlag values). */
    const std::vector<uint8_t>& Flags() const { return m_flags; }
    /* Last compute call's deformation: num_pois x (u, ux, uy, v, vx, vy). */
    const std::vector<real_t>& Deformation() const { return m_p6; }

protected:
    void reset_ref(const ImageView& im) {
        detail::check(twdic_icgn_reset_ref(m_h, im.data, im.step, detail::mem_of(im)), "ResetRefImg");
    }
    twdic_params m_prm;
    twdic_icgn* m_h = nullptr;
    int_t m_iPOINumber = 0;
    std::vector<uint8_t> m_flags;
    std::vector<real_t> m_p6;
};

/* ---------------------------------------------------------- ICGN2D_CPU -- */
class ICGN2D_CPU : public ICGN2D {
public:
    ICGN2D_CPU(int_t iImgWidth, int_t iImgHeight, int_t iStartX, int_t iStartY, int_t iROIWidth, int_t iROIHeight,
               int_t iSubsetX, int_t iSubsetY, int_t iNumberX, int_t iNumberY, int_t iNumIterations, real_t fDeltaP,
               ICGN2DInterpolationFLag Iflag, paDICThreadFlag /*Tflag*/)
        : ICGN2D(iImgWidth, iImgHeight, iStartX, iStartY, iROIWidth, iROIHeight, iSubsetX, iSubsetY, iNumberX,
                 iNumberY, iNumIterations, fDeltaP) {
        detail::check_ctor(twdic_icgn_set_interpolation(m_h, Iflag == ICGN2DInterpolationFLag::BicubicSpline
                                                                ? TWDIC_INTERP_BSPLINE
                                                                : TWDIC_INTERP_BICUBIC),
                           "interpolation");
    }
    ICGN2D_CPU(const ImageView& refImg, int_t iImgWidth, int_t iImgHeight, int_t iStartX, int_t iStartY,
               int_t iROIWidth, int_t iROIHeight, int_t iSubsetX, int_t iSubsetY, int_t iNumberX, int_t iNumberY,
               int_t iNumIterations, real_t fDeltaP, ICGN2DInterpolationFLag Iflag, paDICThreadFlag Tflag)
        : ICGN2D_CPU(iImgWidth, iImgHeight, iStartX, iStartY, iROIWidth, iROIHeight, iSubsetX, iSubsetY, iNumberX,
                     iNumberY, iNumIterations, fDeltaP, Iflag, Tflag) {
        reset_ref(refImg);
    }

    void ResetRefImg(const ImageView& refImg) override { reset_ref(refImg); }
    void SetTarImg(const ImageView& tarImg) override { m_tar = tarImg; }

    /* fU, fV: in/out host arrays; iNumIterations: out; iPOIpos: (y, x) pairs. */
    void ICGN2D_Algorithm(real_t* fU, real_t* fV, int* iNumIterations, int* iPOIpos, const ImageView& tarImg) {
        run(fU, fV, iNumIterations, iPOIpos, tarImg, 0, m_iPOINumber);
    }
    void ICGN2D_Algorithm(real_t* fU, real_t* fV, int* iNumIterations, int* iPOIpos, const ImageView& tarImg,
                          float& fPrecomputeTime, float& fICGNTime) {
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0);
        run(fU, fV, iNumIterations, iPOIpos, tarImg, 0, m_iPOINumber);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        fPrecomputeTime = 0.f;  // inside the device call
        fICGNTime = ms;
    }
    /* The reference's [head, tail) overload computes all POIs
     * (TW_paDIC_ICGN2D_CPU.cpp:198-254); so does this one. */
    void ICGN2D_Algorithm(real_t* fU, real_t* fV, int* iNumIterations, int* iPOIpos, const ImageView& tarImg,
                          int_t /*head*/, int_t /*tail*/) {
        run(fU, fV, iNumIterations, iPOIpos, tarImg, 0, m_iPOINumber);
    }

private:
    void run(real_t* fU, real_t* fV, int* iters, int* poi, const ImageView& tar, int, int) {
        m_flags.assign((size_t)m_iPOINumber, 0);
        m_p6.assign(6 * (size_t)m_iPOINumber, 0.f);
        detail::check(twdic_icgn_compute(m_h, tar.data, tar.step, poi, detail::mem_of(tar), fU, fV, m_p6.data(),
                                         iters, m_flags.data(), TWDIC_MEM_HOST),
                      "ICGN2D_Algorithm");
    }
    ImageView m_tar;
};

/* ------------------------------------------------------------ cuICGN2D -- */
class cuICGN2D : public ICGN2D {
public:
    cuICGN2D(int_t iImgWidth, int_t iImgHeight, int_t iStartX, int_t iStartY, int_t iROIWidth, int_t iROIHeight,
             int_t iSubsetX, int_t iSubsetY, int_t iNumberX, int_t iNumberY, int_t iNumIterations, real_t fDeltaP,
             ICGN2DInterpolationFLag Iflag)
        : ICGN2D(iImgWidth, iImgHeight, iStartX, iStartY, iROIWidth, iROIHeight, iSubsetX, iSubsetY, iNumberX,
                 iNumberY, iNumIterations, fDeltaP) {
        detail::check_ctor(twdic_icgn_set_interpolation(m_h, Iflag == ICGN2DInterpolationFLag::BicubicSpline
                                                                ? TWDIC_INTERP_BSPLINE
                                                                : TWDIC_INTERP_BICUBIC),
                           "interpolation");
    }

    /* Device reference image, already filled (copied into the handle). */
    void cuInitialize(const uchar1* d_fRefImg) {
        reset_ref(ImageView(reinterpret_cast<const unsigned char*>(d_fRefImg), m_prm.img_width, m_prm.img_height,
                            m_prm.img_width, true));
    }
    /* Device target and POIs; d_fU, d_fV in/out device arrays. */
    void cuCompute(const uchar1* d_fTarImg, const int_t* d_iPOIXY, real_t* d_fU, real_t* d_fV) {
        detail::check(twdic_icgn_compute(m_h, reinterpret_cast<const uint8_t*>(d_fTarImg), m_prm.img_width,
                                         d_iPOIXY, TWDIC_MEM_DEVICE, d_fU, d_fV, nullptr, nullptr, nullptr,
                                         TWDIC_MEM_DEVICE),
                      "cuCompute");
    }
    void cuFinalize() {}
    void Initialize(const ImageView& refImg) { reset_ref(refImg); }
    void ResetRefImg(const ImageView& refImg) override { reset_ref(refImg); }
    void SetTarImg(const ImageView& tarImg) override { m_tar = tarImg; }

private:
    ImageView m_tar;
};

}  // namespace paDIC
}  // namespace TW

#endif  // TW_DIC_HPP
