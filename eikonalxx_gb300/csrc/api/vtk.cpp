// Legacy-VTK writers of the drop-in C++ API: EikonalXX::IO::VTKRectilinearGrid3D/2D and
// VTKLines2D (the reference's src/io/vtkRectilinearGrid3d.cpp, vtkRectilinearGrid2d.cpp,
// vtkLines2d.cpp), used by Model3D/Model2D::writeVTK, Solver2D::writeVTK and
// Ray::GradientTracer2D::writeVTK.  Host code: the fields are already on the host when a
// caller writes them.
//
// The file layout is the reference's, so files open the same way in ParaView or VisIt:
//   # vtk DataFile Version 3.0 / title (blanks -> underscores; "vtk_dataset" if empty) /
//   BINARY or ASCII / DATASET RECTILINEAR_GRID / DIMENSIONS nx ny nz /
//   X_, Y_, Z_COORDINATES n float (z written as -(z0 + iz dz), depth positive down) /
//   POINT_DATA n, then SCALARS name float 1 + LOOKUP_TABLE default, VECTORS name float /
//   CELL_DATA n, then SCALARS name float 1 + LOOKUP_TABLE default.
// Binary values are big-endian IEEE float32, each block followed by a newline.  Every
// SCALARS section carries its LOOKUP_TABLE line, as the legacy format requires.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "eikonalxx/geometry2d.hpp"
#include "eikonalxx/geometry3d.hpp"
#include "eikonalxx/io/vtkLines2d.hpp"
#include "eikonalxx/io/vtkRectilinearGrid2d.hpp"
#include "eikonalxx/io/vtkRectilinearGrid3d.hpp"

namespace {

std::string underscored(const std::string &s, const char *fallback) {
    if (s.empty()) return fallback;
    std::string r = s;
    for (char &c : r)
        if (std::isspace(static_cast<unsigned char>(c))) c = '_';
    return r;
}

// One legacy-VTK file being written: header lines, float blocks and the section state.
class LegacyFile {
public:
    void open(const std::string &fileName, const std::string &title, bool binary) {
        close();
        const auto parent = std::filesystem::path(fileName).parent_path();
        if (!parent.empty() && !std::filesystem::exists(parent)) std::filesystem::create_directories(parent);
        out_.open(fileName, std::ios::out | std::ios::trunc | std::ios::binary);
        if (!out_) throw std::runtime_error("Could not open " + fileName + " for writing");
        binary_ = binary;
        points_ = cells_ = false;
        line("# vtk DataFile Version 3.0");
        line(underscored(title, "vtk_dataset"));
        line(binary ? "BINARY" : "ASCII");
    }
    bool isOpen() const noexcept { return out_.is_open(); }
    void close() noexcept {
        if (out_.is_open()) out_.close();
    }
    void line(const std::string &s) { out_ << s << '\n'; }
    // values as float32: big-endian binary (byte order fixed, whatever the host's), or one
    // value per line in ASCII
    void block(const std::vector<float> &v) {
        if (binary_) {
            std::vector<unsigned char> b(4 * v.size());
            for (size_t i = 0; i < v.size(); ++i) {
                std::uint32_t u;
                std::memcpy(&u, &v[i], 4);
                b[4 * i] = static_cast<unsigned char>(u >> 24);
                b[4 * i + 1] = static_cast<unsigned char>(u >> 16);
                b[4 * i + 2] = static_cast<unsigned char>(u >> 8);
                b[4 * i + 3] = static_cast<unsigned char>(u);
            }
            out_.write(reinterpret_cast<const char *>(b.data()), static_cast<std::streamsize>(b.size()));
            out_ << '\n';
        } else {
            std::ostringstream os;
            os << std::setprecision(std::numeric_limits<float>::max_digits10);
            for (float x : v) os << x << '\n';
            out_ << os.str();
        }
    }
    void grid(int nx, int ny, int nz, const std::vector<float> &x, const std::vector<float> &y,
              const std::vector<float> &z) {
        line("DATASET RECTILINEAR_GRID");
        line("DIMENSIONS " + std::to_string(nx) + " " + std::to_string(ny) + " " + std::to_string(nz));
        line("X_COORDINATES " + std::to_string(x.size()) + " float");
        block(x);
        line("Y_COORDINATES " + std::to_string(y.size()) + " float");
        block(y);
        line("Z_COORDINATES " + std::to_string(z.size()) + " float");
        block(z);
    }
    void scalars(bool nodal, size_t n, const std::string &name, const std::vector<float> &v) {
        section(nodal, n);
        line("SCALARS " + underscored(name, "dataset") + " float 1");
        line("LOOKUP_TABLE default");
        block(v);
    }
    void vectors(size_t n, const std::string &name, const std::vector<float> &v) {
        section(true, n);
        line("VECTORS " + underscored(name, "vector_dataset") + " float");
        block(v);
    }

private:
    void section(bool nodal, size_t n) {
        if (!isOpen()) throw std::runtime_error("File not open for writing");
        bool &done = nodal ? points_ : cells_;
        if (!done) line(std::string(nodal ? "POINT_DATA " : "CELL_DATA ") + std::to_string(n));
        done = true;
    }
    std::ofstream out_;
    bool binary_ = true, points_ = false, cells_ = false;
};

std::vector<float> axis(int n, double o, double d, bool depth) {
    std::vector<float> a(n);
    for (int i = 0; i < n; ++i) {
        const float v = static_cast<float>(o) + static_cast<float>(d) * static_cast<float>(i);
        a[i] = depth ? -v : v;
    }
    return a;
}

// A 3D array (cells or nodes, n1 x n2 x n3 along x, y, z) into natural order (x fastest)
// as float32; XYZ-ordered input (z fastest) is transposed.
template <class T>
std::vector<float> natural3(const T *data, int n1, int n2, int n3, bool xyz) {
    if (!data) throw std::invalid_argument("data is NULL");
    std::vector<float> v(static_cast<size_t>(n1) * n2 * n3);
    for (int k = 0; k < n3; ++k)
        for (int j = 0; j < n2; ++j)
            for (int i = 0; i < n1; ++i) {
                const size_t dst = (static_cast<size_t>(k) * n2 + j) * n1 + i;
                const size_t src = xyz ? (static_cast<size_t>(i) * n2 + j) * n3 + k : dst;
                v[dst] = static_cast<float>(data[src]);
            }
    return v;
}

}  // namespace

namespace EikonalXX::IO {

// ------------------------------------------------------------------------- 3D

class VTKRectilinearGrid3D::VTKRectilinearGrid3DImpl {
public:
    LegacyFile file;
    int nx = 0, ny = 0, nz = 0;
};

VTKRectilinearGrid3D::VTKRectilinearGrid3D() : pImpl(std::make_unique<VTKRectilinearGrid3DImpl>()) {}
VTKRectilinearGrid3D::~VTKRectilinearGrid3D() = default;

void VTKRectilinearGrid3D::open(const std::string &fileName, const Geometry3D &g, const std::string &title,
                                const bool writeBinary) {
    close();
    // the accessors throw std::runtime_error / std::invalid_argument on an incomplete geometry
    const int nx = g.getNumberOfGridPointsInX(), ny = g.getNumberOfGridPointsInY(), nz = g.getNumberOfGridPointsInZ();
    const auto x = axis(nx, g.getOriginInX(), g.getGridSpacingInX(), false);
    const auto y = axis(ny, g.getOriginInY(), g.getGridSpacingInY(), false);
    const auto z = axis(nz, g.getOriginInZ(), g.getGridSpacingInZ(), true);
    pImpl->file.open(fileName, title, writeBinary);
    pImpl->file.grid(nx, ny, nz, x, y, z);
    pImpl->nx = nx; pImpl->ny = ny; pImpl->nz = nz;
}
bool VTKRectilinearGrid3D::isOpen() const noexcept { return pImpl->file.isOpen(); }
void VTKRectilinearGrid3D::close() noexcept { pImpl->file.close(); }

template <typename T>
void VTKRectilinearGrid3D::writeNodalDataset(const std::string &name, const T *data, const Ordering3D ordering) const {
    const auto &p = *pImpl;
    const auto v = natural3(data, p.nx, p.ny, p.nz, ordering == Ordering3D::XYZ);
    pImpl->file.scalars(true, v.size(), name, v);
}
template <typename T>
void VTKRectilinearGrid3D::writeCellularDataset(const std::string &name, const T *data,
                                                const Ordering3D ordering) const {
    const auto &p = *pImpl;
    const auto v = natural3(data, p.nx - 1, p.ny - 1, p.nz - 1, ordering == Ordering3D::XYZ);
    pImpl->file.scalars(false, v.size(), name, v);
}
template void VTKRectilinearGrid3D::writeNodalDataset(const std::string &, const float *, Ordering3D) const;
template void VTKRectilinearGrid3D::writeNodalDataset(const std::string &, const double *, Ordering3D) const;
template void VTKRectilinearGrid3D::writeCellularDataset(const std::string &, const float *, Ordering3D) const;
template void VTKRectilinearGrid3D::writeCellularDataset(const std::string &, const double *, Ordering3D) const;

// ------------------------------------------------------------------------- 2D

class VTKRectilinearGrid2D::VTKRectilinearGrid2DImpl {
public:
    LegacyFile file;
    int nx = 0, nz = 0;
};

VTKRectilinearGrid2D::VTKRectilinearGrid2D() : pImpl(std::make_unique<VTKRectilinearGrid2DImpl>()) {}
VTKRectilinearGrid2D::~VTKRectilinearGrid2D() = default;

void VTKRectilinearGrid2D::open(const std::string &fileName, const Geometry2D &g, const std::string &title,
                                const bool writeBinary) {
    close();
    const int nx = g.getNumberOfGridPointsInX(), nz = g.getNumberOfGridPointsInZ();
    const auto x = axis(nx, g.getOriginInX(), g.getGridSpacingInX(), false);
    const auto z = axis(nz, g.getOriginInZ(), g.getGridSpacingInZ(), true);
    pImpl->file.open(fileName, title, writeBinary);
    pImpl->file.grid(nx, 1, nz, x, std::vector<float>(1, 0.0f), z);
    pImpl->nx = nx; pImpl->nz = nz;
}
bool VTKRectilinearGrid2D::isOpen() const noexcept { return pImpl->file.isOpen(); }
void VTKRectilinearGrid2D::close() noexcept { pImpl->file.close(); }

template <typename T>
void VTKRectilinearGrid2D::writeNodalDataset(const std::string &name, const T *data, const Ordering2D ordering) const {
    const auto &p = *pImpl;
    const auto v = natural3(data, p.nx, 1, p.nz, ordering == Ordering2D::XZ);
    pImpl->file.scalars(true, v.size(), name, v);
}
template <typename T>
void VTKRectilinearGrid2D::writeNodalVectorDataset(const std::string &name, const T *data,
                                                   const Ordering2D ordering) const {
    if (!data) throw std::invalid_argument("data is NULL");
    const auto &p = *pImpl;
    const size_t n = static_cast<size_t>(p.nx) * p.nz;
    std::vector<float> v(3 * n);
    for (int iz = 0; iz < p.nz; ++iz)
        for (int ix = 0; ix < p.nx; ++ix) {
            const size_t dst = static_cast<size_t>(iz) * p.nx + ix;
            const size_t src = ordering == Ordering2D::XZ ? static_cast<size_t>(ix) * p.nz + iz : dst;
            v[3 * dst] = static_cast<float>(data[2 * src]);
            v[3 * dst + 1] = 0.0f;
            v[3 * dst + 2] = static_cast<float>(data[2 * src + 1]);
        }
    pImpl->file.vectors(n, name, v);
}
template <typename T>
void VTKRectilinearGrid2D::writeCellularDataset(const std::string &name, const T *data,
                                                const Ordering2D ordering) const {
    const auto &p = *pImpl;
    const auto v = natural3(data, p.nx - 1, 1, p.nz - 1, ordering == Ordering2D::XZ);
    pImpl->file.scalars(false, v.size(), name, v);
}
template void VTKRectilinearGrid2D::writeNodalDataset(const std::string &, const float *, Ordering2D) const;
template void VTKRectilinearGrid2D::writeNodalDataset(const std::string &, const double *, Ordering2D) const;
template void VTKRectilinearGrid2D::writeNodalVectorDataset(const std::string &, const float *, Ordering2D) const;
template void VTKRectilinearGrid2D::writeNodalVectorDataset(const std::string &, const double *, Ordering2D) const;
template void VTKRectilinearGrid2D::writeCellularDataset(const std::string &, const float *, Ordering2D) const;
template void VTKRectilinearGrid2D::writeCellularDataset(const std::string &, const double *, Ordering2D) const;

// ------------------------------------------------------------------ 2D lines

class VTKLines2D::VTKLines2DImpl {
public:
    LegacyFile file;
};

VTKLines2D::VTKLines2D() : pImpl(std::make_unique<VTKLines2DImpl>()) {}
VTKLines2D::~VTKLines2D() = default;

void VTKLines2D::open(const std::string &fileName, const EikonalXX::Geometry2D &, const std::string &title) {
    close();
    pImpl->file.open(fileName, title, false);
    pImpl->file.line("DATASET POLYDATA");
}
bool VTKLines2D::isOpen() const noexcept { return pImpl->file.isOpen(); }
void VTKLines2D::close() noexcept { pImpl->file.close(); }

void VTKLines2D::write(const std::vector<std::vector<std::pair<double, double>>> &polygons) const {
    if (!isOpen()) throw std::runtime_error("File not open");
    size_t nPoints = 0;
    for (const auto &p : polygons) nPoints += p.size();
    std::ostringstream os;
    os << std::setprecision(std::numeric_limits<double>::max_digits10);
    os << "POINTS " << nPoints << " float\n";
    for (const auto &p : polygons)
        for (const auto &q : p) os << q.first << " 0 " << -q.second << '\n';
    os << "LINES " << polygons.size() << " " << nPoints + polygons.size() << '\n';
    size_t k = 0;
    for (const auto &p : polygons) {
        os << p.size();
        for (size_t j = 0; j < p.size(); ++j) os << ' ' << k++;
        os << '\n';
    }
    pImpl->file.line(os.str().substr(0, os.str().size() - 1));
}

}  // namespace EikonalXX::IO
