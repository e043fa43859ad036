// Matrix::D2D / Matrix::D3D binary files (source/Glioma/Matrix.h:26-35, 609-664):
// int header {1234, dim, nx, ny[, nz]}, int type id (0 double, 1 float, 2 int),
// then the elements, x fastest.
#pragma once
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

namespace gbgcli {

struct Matrix {
    int dim = 0;
    int nx = 0, ny = 0, nz = 1;
    std::vector<double> data;
    double operator()(int i, int j) const { return data[(size_t)i + (size_t)j * nx]; }
    double operator()(int i, int j, int k) const { return data[(size_t)i + ((size_t)j + (size_t)k * ny) * nx]; }
};

inline Matrix read_matrix(const std::string &path, int dim) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("ERROR while opening " + path);
    int hdr[2];
    Matrix m;
    if (std::fread(hdr, sizeof(int), 2, f) != 2 || hdr[0] != 1234 || hdr[1] != dim) {
        std::fclose(f);
        throw std::runtime_error("bad matrix header in " + path);
    }
    int sz[3] = {0, 0, 1};
    int tid = -1;
    if (std::fread(sz, sizeof(int), dim, f) != (size_t)dim || std::fread(&tid, sizeof(int), 1, f) != 1) {
        std::fclose(f);
        throw std::runtime_error("truncated matrix header in " + path);
    }
    m.dim = dim;
    m.nx = sz[0];
    m.ny = sz[1];
    m.nz = dim == 3 ? sz[2] : 1;
    const size_t n = (size_t)m.nx * m.ny * m.nz;
    m.data.resize(n);
    bool ok = true;
    if (tid == 0) {
        ok = std::fread(m.data.data(), sizeof(double), n, f) == n;
    } else if (tid == 1) {
        std::vector<float> t(n);
        ok = std::fread(t.data(), sizeof(float), n, f) == n;
        for (size_t i = 0; i < n; ++i) m.data[i] = t[i];
    } else if (tid == 2) {
        std::vector<int> t(n);
        ok = std::fread(t.data(), sizeof(int), n, f) == n;
        for (size_t i = 0; i < n; ++i) m.data[i] = t[i];
    } else {
        ok = false;
    }
    std::fclose(f);
    if (!ok) throw std::runtime_error("bad or truncated matrix data in " + path);
    return m;
}

inline void write_d3d(const std::string &path, int nx, int ny, int nz, const std::vector<double> &data) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("ERROR while opening " + path);
    const int hdr[6] = {1234, 3, nx, ny, nz, 0};
    std::fwrite(hdr, sizeof(int), 6, f);
    std::fwrite(data.data(), sizeof(double), data.size(), f);
    std::fclose(f);
}

// -key value command-line arguments (the reference's ArgumentParser keys)
struct Args {
    int argc;
    char **argv;
    const char *find(const char *key) const {
        for (int i = 1; i + 1 < argc; ++i)
            if (std::string(argv[i]) == key) return argv[i + 1];
        return nullptr;
    }
    int as_int(const char *key, int def) const {
        const char *v = find(key);
        return v ? std::atoi(v) : def;
    }
    double as_double(const char *key, double def) const {
        const char *v = find(key);
        return v ? std::atof(v) : def;
    }
    std::string as_string(const char *key, const std::string &def) const {
        const char *v = find(key);
        return v ? std::string(v) : def;
    }
};

}  // namespace gbgcli
