// The reference's seven exports (isar_imaging_export.h) on top of the C ABI:
// .wbd ingest (dataParsing / dataExtracting, common.cu:750-1191), process-wide
// workspace (imagingMemInit / imagingMemDest, isar_imaging_export.cpp:121-279)
// and one image per call (isarMainSingle, isar_imaging_export.cpp:208-212).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <regex>
#include <string>
#include <vector>

#include "../../include/isar_gb300.h"
#include "../../include/isar_imaging_export.h"

namespace fs = std::filesystem;

namespace {

constexpr float kPiF = 3.14159265358979f;
constexpr int kRangeCut = 512;

// Process-wide state of the export layer (the reference keeps the same in
// globals, isar_imaging_export.cpp:4-35).
struct ExportState {
    std::vector<std::string> files;   // matching .wbd files
    int data_type = 0;
    long long fc = 0, band_width = 0, Fs = 0;
    double Tp = 0.0;
    int echo_num = 0, range_num = 0;
    isar_ctx* ctx = nullptr;
    float* d_pp[2] = {nullptr, nullptr};   // ping-pong raw windows
    int cur = -1;                          // which d_pp holds the current window
    int win_type = 0;                      // data type the windows were extracted as
    double* d_vel = nullptr;
    float* d_img = nullptr;
    // IFDS: raw int16 samples and per-pulse velocities of the new pulses
    int16_t* d_ad = nullptr;
    double* d_pcvel = nullptr;
    size_t ad_len = 0;
};

ExportState& st()
{
    static ExportState s;
    return s;
}

void report(const char* where)
{
    char msg[512];
    isar_get_last_error(msg, sizeof(msg));
    std::cout << "[" << where << "/ERROR] " << msg << std::endl;
}

// getTurnAngle (common.cu:983-995), float as written.
float turn_angle(float a1, float p1, float a2, float p2)
{
    const float v1[3] = {std::sin(p1 / 180 * kPiF), std::cos(p1 / 180 * kPiF) * std::cos(a1 / 180 * kPiF),
                         std::cos(p1 / 180 * kPiF) * std::sin(a1 / 180 * kPiF)};
    const float v2[3] = {std::sin(p2 / 180 * kPiF), std::cos(p2 / 180 * kPiF) * std::cos(a2 / 180 * kPiF),
                         std::cos(p2 / 180 * kPiF) * std::sin(a2 / 180 * kPiF)};
    return std::acos(v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2]) / kPiF * 180;
}

// interpolate (common.cu:998-1020): piecewise linear, clamped at the ends.
float interpolate(const std::vector<int>& xd, const std::vector<float>& yd, int x)
{
    const int size = (int)xd.size();
    int i = 0;
    if (x >= xd[size - 2]) {
        i = size - 2;
    } else {
        while (x > xd[i + 1]) ++i;
    }
    const float xL = (float)xd[i], xR = (float)xd[i + 1];
    float yL = yd[i], yR = yd[i + 1];
    if (x < xL) yR = yL;
    if (x > xR) yL = yR;
    const float dydx = (yR - yL) / (xR - xL);
    return yL + dydx * ((float)x - xL);
}

// turnAngleLine (common.cu:902-980): accumulated turn angle per pulse, blocks
// split where the pitching jumps by more than 0.2 degree, 20-pulse steps
// linearly interpolated in blocks of 21 pulses or more.  As in the reference
// the interpolation knots are read at absolute indices x (not block-relative).
// Blocks too short for two knots (21..39 pulses, where the reference indexes
// before its knot vector) keep their uninterpolated values.
void turn_angle_line(std::vector<float>* ta, const std::vector<float>& az, const std::vector<float>& pit)
{
    const int P = (int)pit.size();
    std::vector<int> idx;
    for (int i = 0; i < P - 1; ++i)
        if (std::abs(pit[i + 1] - pit[i]) > 0.2) idx.push_back(i);
    std::vector<int> beg, end;
    beg.push_back(0);
    for (int v : idx) beg.push_back(v + 1);
    for (int v : idx) end.push_back(v);
    end.push_back(P - 1);
    const int nb = (int)beg.size();
    ta->assign(P, 0.0f);
    for (int b = 0; b < nb; ++b) {
        const int n = end[b] - beg[b] + 1;
        const int stride = (n < 21) ? 1 : 20;
        for (int i = stride; i < n; i += stride) {
            const int c = beg[b] + i;
            (*ta)[c] = (*ta)[c - stride] + turn_angle(az[c - stride], pit[c - stride], az[c], pit[c]);
        }
        for (float& v : *ta) v = std::abs(v);
        if (n >= 21) {
            std::vector<int> x;
            for (int i = 0; i + stride <= n; i += stride) x.push_back(i);
            if (x.size() >= 2) {
                std::vector<float> y;
                for (int xi : x) y.push_back((*ta)[xi]);
                std::vector<float> interp(n);
                for (int i = 0; i < n; ++i) interp[i] = interpolate(x, y, i);
                std::copy(interp.begin(), interp.end(), ta->begin() + beg[b]);
            }
        }
        if (b > 0)
            for (int i = beg[b]; i <= end[b]; ++i) (*ta)[i] += (*ta)[end[b - 1]];
    }
}

}  // namespace

extern "C" {

DLL_EXPORT_API int gpuDevInit()
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return EXIT_FAILURE;
    int best = 0, best_sm = -1;
    for (int d = 0; d < n; ++d) {
        int sm = 0;
        cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, d);
        if (sm > best_sm) {
            best_sm = sm;
            best = d;
        }
    }
    return cudaSetDevice(best) == cudaSuccess ? EXIT_SUCCESS : EXIT_FAILURE;
}

DLL_EXPORT_API int dataParsing(vec1D_DBL* dataN, vec1D_FLT* turnAngle, int* frame_len, int* frame_num,
                               const std::string& dir_path, const int& polar_type, const int& data_type)
{
    ExportState& s = st();
    s.files.clear();
    s.data_type = data_type;
    // ioInit (common.cu:750-793)
    std::error_code ec;
    const std::string dir = fs::absolute(dir_path, ec).string();
    if (!fs::is_directory(dir, ec)) {
        std::cout << "[ioInit/ERROR] Invalid directory path!\n";
        return EXIT_FAILURE;
    }
    std::string pat;
    if (data_type == ISAR_DATA_IFDS) pat = polar_type == 0 ? R"(.*01_1100.*\.wbd)" : R"(.*01_1101.*\.wbd)";
    else if (data_type == ISAR_DATA_STRETCH) pat = polar_type == 0 ? R"(.*00_1100\.wbd)" : R"(.*00_1101\.wbd)";
    else {
        std::cout << "[ioInit/ERROR] Invalid data type!\n";
        return EXIT_FAILURE;
    }
    const std::regex re(pat);
    for (const auto& e : fs::directory_iterator(dir)) {
        const std::string name = e.path().string();
        if (e.is_regular_file() && std::regex_match(name, re)) s.files.push_back(name);
    }
    std::sort(s.files.begin(), s.files.end());   // the reference keeps directory order
    if (s.files.empty()) {
        std::cout << "[ioInit/ERROR] No valid file in the given directory!\n";
        return EXIT_FAILURE;
    }
    // getSystemParas (common.cu:796-833)
    std::ifstream f0(s.files[0], std::ios::binary);
    uint32_t h[36] = {};
    if (!f0.read(reinterpret_cast<char*>(h), sizeof(h))) {
        std::cout << "[getSystemParas/WARN] Cannot open file " << s.files[0] << " !\n";
        return EXIT_FAILURE;
    }
    *frame_len = (int)h[4] * 4;
    s.fc = (long long)h[12] * 1000000LL;
    s.band_width = (long long)h[13] * 1000000LL;
    s.Tp = (double)h[15] / 1000000.0;
    s.Fs = (long long)(h[17] % (1u << 16)) * 1000000LL;
    if (data_type == ISAR_DATA_IFDS) s.Fs /= 2;
    if (*frame_len <= 0) {
        std::cout << "[getSystemParas/ERROR] frame length 0\n";
        return EXIT_FAILURE;
    }
    *frame_num = (int)(fs::file_size(s.files[0]) / (uintmax_t)*frame_len);
    // readKuIFDSAllNB (common.cu:836-899)
    const int total = *frame_num * (int)s.files.size();
    dataN->assign((size_t)total * 4, 0.0);
    std::vector<float> az(total), pit(total);
    std::vector<std::ifstream> ifs;
    for (const auto& p : s.files) ifs.emplace_back(p, std::ios::binary);
    const double p31 = std::pow(2.0, 31), p32 = std::pow(2.0, 32), p24 = std::pow(2.0, 24);
    for (int i = 0; i < total; ++i) {
        const int fi = i / *frame_num;
        uint32_t nav[11] = {};
        ifs[fi].seekg((std::streamoff)(i - fi * *frame_num) * *frame_len + 48, std::ios::beg);
        ifs[fi].read(reinterpret_cast<char*>(nav), sizeof(nav));
        const double range = (double)nav[7] * 0.1;
        double vel = (double)nav[8], azi = (double)nav[9], pitch = (double)nav[10];
        vel = (vel - (vel > p31 ? p32 : 0)) * 0.1;
        azi = (azi - (azi > p31 ? p32 : 0)) * (360.0 / p24);
        azi += (azi < 0 ? 360.0 : 0);
        pitch = (pitch - (pitch > p31 ? p32 : 0)) * (360.0 / p24);
        pitch += (pitch < 0 ? 360.0 : 0);
        (*dataN)[i] = range;
        (*dataN)[i + (size_t)total] = vel;
        (*dataN)[i + 2 * (size_t)total] = azi;
        (*dataN)[i + 3 * (size_t)total] = pitch;
        az[i] = (float)azi;
        pit[i] = (float)pitch;
    }
    turn_angle_line(turnAngle, az, pit);
    return EXIT_SUCCESS;
}

DLL_EXPORT_API void imagingMemInit(vec1D_FLT* img, vec1D_INT* dataWFileSn, vec1D_DBL* dataNOut,
                                   vec1D_FLT* turnAngleOut, vec1D_COM_FLT* dataW, const int& window_len,
                                   const int& frame_len, const int& data_type, const bool& if_hpc,
                                   const bool& if_hrrp)
{
    (void)if_hpc;
    (void)if_hrrp;
    ExportState& s = st();
    const int M = window_len;
    const int N = (data_type == ISAR_DATA_STRETCH) ? (frame_len - 256) / 4 : 4096;   // RANGE_NUM_IFDS_PC
    // guards of isar_imaging_export.cpp:144-155
    if (M > 1024) {
        std::cout << "[main/WARN] echo_num > MAX_THREAD_PER_BLOCK: 1024, please double-check the data, then "
                     "reconfiguring the parameters."
                  << std::endl;
        return;
    }
    if (N < kRangeCut) {
        std::cout << "[main/WARN] range_num < paras.range_num_cut: 512, please double-check the data or optimize "
                     "process of cutRangeProfile()."
                  << std::endl;
        return;
    }
    if (N < M) {
        std::cout << "[main/WARN] range_num < echo_num, please double-check the data." << std::endl;
        return;
    }
    img->resize((size_t)M * kRangeCut);
    dataWFileSn->resize(M);
    dataNOut->resize((size_t)M * 4);
    turnAngleOut->resize(M);
    if (data_type == ISAR_DATA_STRETCH) dataW->resize((size_t)M * N);
    if (s.ctx) {
        isar_destroy(s.ctx);
        s.ctx = nullptr;
    }
    isar_radar r{};
    r.echo_num = M;
    r.range_num = N;
    r.band_width = s.band_width;
    r.fc = s.fc;
    r.Tp = s.Tp;
    r.Fs = s.Fs;
    r.data_type = data_type;
    int dev = 0;
    cudaGetDevice(&dev);
    if (isar_create(&s.ctx, &r, dev, nullptr) != ISAR_OK) {
        report("imagingMemInit");
        return;
    }
    s.echo_num = M;
    s.range_num = N;
    s.cur = -1;
    const size_t MN = (size_t)M * N;
    bool ok = cudaMalloc(&s.d_pp[0], MN * 2 * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&s.d_pp[1], MN * 2 * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&s.d_vel, M * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&s.d_img, (size_t)M * kRangeCut * sizeof(float)) == cudaSuccess;
    if (!ok) std::cout << "[imagingMemInit/ERROR] device allocation failed" << std::endl;
    else cudaMemset(s.d_vel, 0, M * sizeof(double));
}

DLL_EXPORT_API int dataExtracting(vec1D_INT* dataWFileSn, vec1D_DBL* dataNOut, vec1D_FLT* turnAngleOut,
                                  vec1D_COM_FLT* dataW, const vec1D_DBL& dataN, const vec1D_FLT& turnAngle,
                                  const int& frame_len, const int& frame_num, const int& sampling_stride,
                                  const int& window_head, const int& window_len, int& imaging_stride,
                                  const int& data_type)
{
    ExportState& s = st();
    if (!s.ctx || !s.d_pp[0]) {
        std::cout << "[dataExtracting/ERROR] imagingMemInit has not succeeded" << std::endl;
        return EXIT_FAILURE;
    }
    if (data_type != ISAR_DATA_STRETCH && data_type != ISAR_DATA_IFDS) {
        std::cout << "[dataExtracting/ERROR] Invalid data type!" << std::endl;
        return EXIT_FAILURE;
    }
    const int M = s.echo_num, N = s.range_num;
    // uniformSampling (common.cu:1165-1185)
    const int total = frame_num * (int)s.files.size();
    for (int i = 0; i < window_len; ++i) (*dataWFileSn)[i] = window_head + i * sampling_stride;
    for (int i = 0; i < window_len; ++i) {
        const int sn = (*dataWFileSn)[i];
        if (sn < 0 || sn >= total) {
            std::cout << "[dataExtracting/ERROR] pulse " << sn << " beyond the " << total << " parsed frames"
                      << std::endl;
            return EXIT_FAILURE;
        }
        for (int j = 0; j < 4; ++j) (*dataNOut)[(size_t)j * window_len + i] = dataN[sn + (size_t)j * total];
        (*turnAngleOut)[i] = std::abs(turnAngle[sn]);
    }
    // ping-pong choice and overlap reuse (isar_imaging_export.cpp:88-105)
    int overlap = 0;
    int next = 0;
    if (s.cur >= 0) {
        next = 1 - s.cur;
        overlap = M - imaging_stride;
        if (overlap < 0) overlap = 0;
        if (overlap > M) overlap = M;
    }
    const int new_len = M - overlap;
    if (s.cur >= 0 && s.win_type != data_type) {
        std::cout << "[dataExtracting/ERROR] data type changed between windows" << std::endl;
        return EXIT_FAILURE;
    }
    s.win_type = data_type;
    // A window row: IFDS, the 4096 complex64 cells of a compressed pulse;
    // STRETCH, the pulse's 2N int16 I/Q samples as read (imaged with
    // ISAR_FLAG_IQ16: half the bytes to copy and to keep).
    const size_t row_bytes = data_type == ISAR_DATA_IFDS ? (size_t)N * 2 * sizeof(float) : (size_t)N * 2 * sizeof(int16_t);
    char* pp_next = reinterpret_cast<char*>(s.d_pp[next]);
    if (overlap > 0 &&
        cudaMemcpy(pp_next, reinterpret_cast<const char*>(s.d_pp[s.cur]) + (size_t)new_len * row_bytes,
                   (size_t)overlap * row_bytes, cudaMemcpyDeviceToDevice) != cudaSuccess) {
        std::cout << "[dataExtracting/ERROR] overlap copy failed" << std::endl;
        return EXIT_FAILURE;
    }
    std::vector<std::ifstream> ifs;
    for (const auto& p : s.files) ifs.emplace_back(p, std::ios::binary);
    const int ad_size = (frame_len - 256) / 2;
    if (data_type == ISAR_DATA_IFDS) {
        // getSignalData IFDS branch (common.cu:1043-1083): every new pulse's
        // int16 samples (byte 256 on) are pulse-compressed into its row of
        // the window (multiThreadIFDS, common.cu:583-604), here all new pulses
        // in one launch.  Velocity of pulse i: dataNOut[echo_num +
        // dataWFileSn[i]] as the reference indexes it (common.cu:602; the file
        // serial number, not the window position).
        const int iq_len = ad_size / 2;
        std::vector<int16_t> h_ad((size_t)new_len * 2 * iq_len);
        std::vector<double> h_v(new_len);
        for (int i = overlap; i < M; ++i) {
            const int sn = (*dataWFileSn)[i];
            const int fi = sn / frame_num;
            const size_t vi = (size_t)M + (size_t)sn;
            if (vi >= dataNOut->size()) {
                std::cout << "[dataExtracting/ERROR] velocity index " << vi << " beyond dataNOut ("
                          << dataNOut->size() << ")" << std::endl;
                return EXIT_FAILURE;
            }
            h_v[i - overlap] = (*dataNOut)[vi];
            ifs[fi].seekg((std::streamoff)(sn - fi * frame_num) * frame_len + 256, std::ios::beg);
            if (!ifs[fi].read(reinterpret_cast<char*>(h_ad.data() + (size_t)(i - overlap) * 2 * iq_len),
                              (std::streamsize)iq_len * 4)) {
                std::cout << "[dataExtracting/ERROR] short read in " << s.files[fi] << std::endl;
                return EXIT_FAILURE;
            }
        }
        if (h_ad.size() > s.ad_len) {
            if (s.d_ad) cudaFree(s.d_ad);
            if (s.d_pcvel) cudaFree(s.d_pcvel);
            s.d_ad = nullptr;
            s.d_pcvel = nullptr;
            s.ad_len = 0;
            if (cudaMalloc(&s.d_ad, h_ad.size() * sizeof(int16_t)) != cudaSuccess ||
                cudaMalloc(&s.d_pcvel, (size_t)M * sizeof(double)) != cudaSuccess) {
                std::cout << "[dataExtracting/ERROR] device allocation failed" << std::endl;
                return EXIT_FAILURE;
            }
            s.ad_len = h_ad.size();
        }
        cudaStream_t cs = (cudaStream_t)isar_stream(s.ctx);
        if (new_len > 0) {
            if (cudaMemcpyAsync(s.d_ad, h_ad.data(), h_ad.size() * sizeof(int16_t), cudaMemcpyHostToDevice, cs) !=
                    cudaSuccess ||
                cudaMemcpyAsync(s.d_pcvel, h_v.data(), (size_t)new_len * sizeof(double), cudaMemcpyHostToDevice,
                                cs) != cudaSuccess) {
                std::cout << "[dataExtracting/ERROR] sample copy failed" << std::endl;
                return EXIT_FAILURE;
            }
            if (isar_pulse_compress(s.ctx, s.d_ad, iq_len, s.d_pcvel, new_len,
                                    reinterpret_cast<float*>(pp_next + (size_t)overlap * row_bytes),
                                    nullptr) != ISAR_OK) {
                report("dataExtracting");
                return EXIT_FAILURE;
            }
        }
        if (cudaStreamSynchronize(cs) != cudaSuccess) {
            std::cout << "[dataExtracting/ERROR] pulse compression failed" << std::endl;
            return EXIT_FAILURE;
        }
        s.cur = next;
        return EXIT_SUCCESS;
    }
    // getSignalData STRETCH branch (common.cu:1085-1106): int16 I/Q at byte
    // 256.  dataW receives the float samples as in the reference; the device
    // window gets the int16 samples themselves.
    std::vector<int16_t> ad((size_t)new_len * 2 * N);
    for (int i = overlap; i < M; ++i) {
        const int sn = (*dataWFileSn)[i];
        const int fi = sn / frame_num;
        int16_t* a = ad.data() + (size_t)(i - overlap) * 2 * N;
        ifs[fi].seekg((std::streamoff)(sn - fi * frame_num) * frame_len + 256, std::ios::beg);
        if (ad_size < 2 * N || !ifs[fi].read(reinterpret_cast<char*>(a), (std::streamsize)2 * N * 2)) {
            std::cout << "[dataExtracting/ERROR] short read in " << s.files[fi] << std::endl;
            return EXIT_FAILURE;
        }
        std::complex<float>* dst = dataW->data() + (size_t)i * N;
        for (int j = 0; j < N; ++j) dst[j] = std::complex<float>(a[2 * j], a[2 * j + 1]);
    }
    if (new_len > 0 &&
        cudaMemcpy(pp_next + (size_t)overlap * row_bytes, ad.data(), (size_t)new_len * row_bytes,
                   cudaMemcpyHostToDevice) != cudaSuccess) {
        std::cout << "[dataExtracting/ERROR] echo copy failed" << std::endl;
        return EXIT_FAILURE;
    }
    if (cudaMemcpy(s.d_vel, dataNOut->data() + M, M * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        std::cout << "[dataExtracting/ERROR] velocity copy failed" << std::endl;
        return EXIT_FAILURE;
    }
    s.cur = next;
    return EXIT_SUCCESS;
}

DLL_EXPORT_API void isarMainSingle(float* h_img, const int& data_type, const int& option_alignment,
                                   const int& option_phase, const bool& if_hrrp, const bool& if_hpc,
                                   const bool& if_mtrc)
{
    (void)option_alignment;
    (void)option_phase;
    ExportState& s = st();
    if (!s.ctx || s.cur < 0) {
        std::cout << "[isarMainSingle/ERROR] no window extracted" << std::endl;
        return;
    }
    (void)data_type;
    int flags = (if_hpc ? ISAR_FLAG_HPC : 0) | (if_mtrc ? ISAR_FLAG_MTRC : 0) | (if_hrrp ? ISAR_FLAG_HRRP : 0);
    if (s.win_type == ISAR_DATA_STRETCH) flags |= ISAR_FLAG_IQ16;   // the window holds int16 samples
    if (isar_image_device(s.ctx, s.d_pp[s.cur], s.d_vel, flags, s.d_img) != ISAR_OK) {
        report("isarMainSingle");
        return;
    }
    if (cudaMemcpyAsync(h_img, s.d_img, (size_t)s.echo_num * kRangeCut * sizeof(float), cudaMemcpyDeviceToHost,
                        (cudaStream_t)isar_stream(s.ctx)) != cudaSuccess ||
        cudaStreamSynchronize((cudaStream_t)isar_stream(s.ctx)) != cudaSuccess)
        std::cout << "[isarMainSingle/ERROR] image copy failed" << std::endl;
}

DLL_EXPORT_API void writeFileFLT(const std::string& outFilePath, const float* data, const size_t& data_size)
{
    // ioOperation::writeFile (common.cu:1228-1242)
    std::ofstream ofs(outFilePath);
    if (!ofs.is_open()) {
        std::cout << "[writeFile/WARN] Cannot open the file: " << outFilePath << std::endl;
        return;
    }
    for (size_t i = 0; i < data_size; ++i) ofs << std::fixed << std::setprecision(5) << data[i] << "\n";
}

DLL_EXPORT_API void imagingMemDest(const int& data_type, const bool& if_hpc, const bool& if_hrrp)
{
    (void)data_type;
    (void)if_hpc;
    (void)if_hrrp;
    ExportState& s = st();
    if (s.ctx) isar_destroy(s.ctx);
    s.ctx = nullptr;
    for (float*& p : s.d_pp) {
        if (p) cudaFree(p);
        p = nullptr;
    }
    if (s.d_vel) cudaFree(s.d_vel);
    if (s.d_img) cudaFree(s.d_img);
    if (s.d_ad) cudaFree(s.d_ad);
    if (s.d_pcvel) cudaFree(s.d_pcvel);
    s.d_vel = nullptr;
    s.d_img = nullptr;
    s.d_ad = nullptr;
    s.d_pcvel = nullptr;
    s.ad_len = 0;
    s.cur = -1;
}

}  // extern "C"
