// io.cpp — file formats around the time step: MatrixMarket vectors and
// matrices (IO::readVector / IO::writeMatrix with fileFormat 1, IO.hpp:21-145;
// model files <ModelFilename>.<parameter>.mtx, seismograms
// <SeismogramFilename>.shot_<n>.<component>.mtx) and SeismicUnix traces
// (SUIO::writeSU, SUIO.hpp:156-262). Host code.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/wave.h"

namespace wave {
void set_global_error(const std::string& msg);
}

namespace {

int err(int code, const std::string& m)
{
    wave::set_global_error(m);
    return code;
}

// SeismicUnix trace header: 240 bytes, the standard field offsets of the SU
// format (tracl at 0 ... ns at 114, dt at 116, d1 at 180, ntr at 204).
struct SuHeader {
    unsigned char b[240];
    void i32(int off, int32_t v) { std::memcpy(b + off, &v, 4); }
    void i16(int off, int16_t v) { std::memcpy(b + off, &v, 2); }
    void u16(int off, uint16_t v) { std::memcpy(b + off, &v, 2); }
    void f32(int off, float v) { std::memcpy(b + off, &v, 4); }
};

} // namespace

extern "C" {

// Reads a MatrixMarket file ("array" or "coordinate", real) as a row-major
// rows x cols matrix. With out == NULL only the dimensions are returned.
int wave_read_mtx(const char* path, float* out, int64_t capacity, int64_t* rows, int64_t* cols)
{
    if (!path || !rows || !cols) return err(WAVE_ERR_ARG, "wave_read_mtx: null argument");
    std::ifstream f(path);
    if (!f.good()) return err(WAVE_ERR_IO, std::string("wave_read_mtx: cannot open ") + path);
    std::string banner;
    std::getline(f, banner);
    if (banner.rfind("%%MatrixMarket", 0) != 0) return err(WAVE_ERR_IO, std::string("wave_read_mtx: not a MatrixMarket file: ") + path);
    const bool coordinate = banner.find("coordinate") != std::string::npos;
    std::string line;
    while (std::getline(f, line))
        if (!line.empty() && line[0] != '%') break;
    std::istringstream hdr(line);
    long long r = 0, c = 0, nnz = 0;
    hdr >> r >> c;
    if (coordinate) hdr >> nnz;
    if (hdr.fail() || r < 0 || c < 0) return err(WAVE_ERR_IO, std::string("wave_read_mtx: bad size line in ") + path);
    *rows = r;
    *cols = c;
    if (!out) return WAVE_OK;
    if (capacity < r * c) return err(WAVE_ERR_ARG, "wave_read_mtx: output too small");
    std::fill(out, out + r * c, 0.0f);
    if (coordinate) {
        for (long long k = 0; k < nnz; ++k) {
            long long i, j;
            double v;
            if (!(f >> i >> j >> v)) return err(WAVE_ERR_IO, std::string("wave_read_mtx: truncated ") + path);
            if (i < 1 || i > r || j < 1 || j > c) return err(WAVE_ERR_IO, std::string("wave_read_mtx: index out of range in ") + path);
            out[(i - 1) * c + (j - 1)] = static_cast<float>(v);
        }
    } else {
        // array format: column-major
        for (long long j = 0; j < c; ++j)
            for (long long i = 0; i < r; ++i) {
                double v;
                if (!(f >> v)) return err(WAVE_ERR_IO, std::string("wave_read_mtx: truncated ") + path);
                out[i * c + j] = static_cast<float>(v);
            }
    }
    return WAVE_OK;
}

// Writes a row-major rows x cols matrix in MatrixMarket array format (a
// vector is rows x 1).
int wave_write_mtx(const char* path, const float* data, int64_t rows, int64_t cols)
{
    if (!path || (!data && rows * cols > 0) || rows < 0 || cols < 0) return err(WAVE_ERR_ARG, "wave_write_mtx: invalid argument");
    std::FILE* f = std::fopen(path, "w");
    if (!f) return err(WAVE_ERR_IO, std::string("wave_write_mtx: cannot create ") + path);
    std::fprintf(f, "%%%%MatrixMarket matrix array real general\n%lld %lld\n", static_cast<long long>(rows), static_cast<long long>(cols));
    for (long long j = 0; j < cols; ++j)
        for (long long i = 0; i < rows; ++i) std::fprintf(f, "%.9g\n", static_cast<double>(data[i * cols + j]));
    const bool ok = std::fclose(f) == 0;
    return ok ? WAVE_OK : err(WAVE_ERR_IO, std::string("wave_write_mtx: write failed for ") + path);
}

// Writes ntr traces of ns samples (row-major) as a SeismicUnix file with the
// trace headers of SUIO::writeSU: positions relative to the source, in
// millimetres with scalel = scalco = -3, depth axis y, sample interval dt.
int wave_write_su(const char* path, const float* data, int64_t ntr, int64_t ns, double dt, const int64_t* rec_idx, int64_t src_idx,
                  int64_t NX, int64_t NY, int64_t NZ, double DH)
{
    if (!path || !data || !rec_idx || ntr < 0 || ns < 1 || ns > 65535 || dt <= 0 || NX < 1 || NY < 1 || NZ < 1)
        return err(WAVE_ERR_ARG, "wave_write_su: invalid argument");
    auto coord = [&](int64_t i, float& x, float& y, float& z) {
        const int64_t yy = i / (NX * NZ), rem = i - yy * NX * NZ, zz = rem / NX, xx = rem - zz * NX;
        x = static_cast<float>(xx) * static_cast<float>(DH);
        y = static_cast<float>(yy) * static_cast<float>(DH);
        z = static_cast<float>(zz) * static_cast<float>(DH);
    };
    std::FILE* f = std::fopen(path, "wb");
    if (!f) return err(WAVE_ERR_IO, std::string("wave_write_su: cannot create ") + path);
    float XS, YS, ZS;
    coord(src_idx, XS, YS, ZS);
    const float xshift = 800.0f, yshift = 800.0f;
    const float dtus = static_cast<float>(dt * 1000000.0);
    const double pi = 3.1415926;
    bool ok = true;
    for (int64_t t = 0; t < ntr && ok; ++t) {
        SuHeader h;
        std::memset(h.b, 0, sizeof(h.b));
        float xr, yr, zr;
        coord(rec_idx[t], xr, yr, zr);
        const float x = xr - XS, y = yr - YS, z = zr - ZS;
        h.i32(0, static_cast<int32_t>(t + 1));                 // tracl
        h.i32(4, 1);                                           // tracr
        h.i32(16, 1);                                          // ep
        h.i32(20, static_cast<int32_t>(ntr));                  // cdp
        h.i16(28, 1);                                          // trid
        h.i32(36, static_cast<int32_t>(std::lround(std::sqrt((XS - xr) * (XS - xr) + (YS - yr) * (YS - yr) + (ZS - zr) * (ZS - zr)) * 1000.0)));
        h.i32(40, static_cast<int32_t>(std::lround(yr * 1000.0)));   // gelev
        h.i32(48, static_cast<int32_t>(std::lround(YS * 1000.0)));   // sdepth
        h.i32(52, static_cast<int32_t>(std::lround(std::atan2(-y, z) * 180 * 1000.0 / pi)));    // gdel
        h.i32(60, static_cast<int32_t>(std::lround(((360.0 / (2.0 * pi)) * std::atan2(x - xshift, y - yshift)) * 1000.0)));  // swdep
        h.i32(64, static_cast<int32_t>(std::lround(std::sqrt(z * z + y * y) * 1000.0)));          // gwdep
        h.i16(68, -3);                                         // scalel
        h.i16(70, -3);                                         // scalco
        h.i32(72, static_cast<int32_t>(std::lround(XS * 1000.0)));   // sx
        h.i32(76, static_cast<int32_t>(std::lround(ZS * 1000.0)));   // sy
        h.i32(80, static_cast<int32_t>(std::lround(xr * 1000.0)));   // gx
        h.i32(84, static_cast<int32_t>(std::lround(zr * 1000.0)));   // gy
        const uint16_t dtu = static_cast<uint16_t>(std::lround(dtus));
        h.u16(114, static_cast<uint16_t>(ns));                 // ns
        h.u16(116, dtu);                                       // dt in microseconds
        h.f32(180, static_cast<float>(dtu) * 1.0e-6f);         // d1
        h.i32(204, static_cast<int32_t>(ntr));                 // ntr
        ok = std::fwrite(h.b, 1, 240, f) == 240 &&
             std::fwrite(data + t * ns, sizeof(float), static_cast<size_t>(ns), f) == static_cast<size_t>(ns);
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? WAVE_OK : err(WAVE_ERR_IO, std::string("wave_write_su: write failed for ") + path);
}

} // extern "C"
