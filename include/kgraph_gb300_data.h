/* kgraph_gb300_data.h - dense data containers and the matrix oracle of the
 * FastKCNA interface (reference: src/kgraph-data.h), for the GB300 library.
 *
 *   Matrix<T>            row-major rows padded to a 32-byte stride; load()
 *                        (raw with skip/gap), load_lshkit(), save_lshkit(),
 *                        hnsw_dataload() (rows stored in HNSW level order).
 *   hnsw_levels()        the level assignment of hnsw_dataload
 *                        (src/kgraph-data.h:179-222): level =
 *                        (int)(-ln U * 1/ln M) with U drawn by
 *                        std::uniform_real_distribution<double>(0, 1) from a
 *                        std::default_random_engine seeded with `seed`, nodes
 *                        ordered by level, highest first, ties by file order.
 *   MatrixOracle<M, D>   IndexOracle + RowSource over a Matrix<float>; the
 *                        host distance D (metric::l2sqr: the canonical
 *                        fused multiply-add chain the device kernels use).
 */
#ifndef KGRAPH_GB300_DATA_H
#define KGRAPH_GB300_DATA_H

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>
#include <fstream>
#include <random>
#include <string>
#include <vector>

#include "kgraph_gb300.h"

#ifndef KGRAPH_MATRIX_ALIGN
#define KGRAPH_MATRIX_ALIGN 32
#endif

namespace kgraph {

namespace metric {
/* squared L2 as one FMA chain over the dimensions in order */
struct l2sqr {
    template <typename T>
    static float apply(T const *a, T const *b, unsigned dim) {
        float r = 0.f;
        for (unsigned i = 0; i < dim; ++i) {
            const float v = float(a[i]) - float(b[i]);
            r = std::fma(v, v, r);
        }
        return r;
    }
    template <typename T>
    static float dot(T const *a, T const *b, unsigned dim) {
        float r = 0.f;
        for (unsigned i = 0; i < dim; ++i) r = std::fma(float(a[i]), float(b[i]), r);
        return r;
    }
    template <typename T>
    static float norm2(T const *a, unsigned dim) {
        return dot(a, a, dim);
    }
};
} // namespace metric

/* Levels of n nodes for an HNSW of M links; out: level per file row,
 * data2file (storage order -> file row), points_num[l] = nodes on level l. */
inline void hnsw_levels(unsigned n, unsigned M, unsigned seed, std::vector<int> &level,
                        std::vector<int> &data2file, std::vector<int> &points_num) {
    std::default_random_engine gen;
    gen.seed(seed);
    const double mult = 1.0 / std::log(1.0 * M);
    level.assign(n, 0);
    int top = 0;
    for (unsigned i = 0; i < n; ++i) {
        std::uniform_real_distribution<double> u(0.0, 1.0);
        level[i] = (int)(-std::log(u(gen)) * mult);
        if (level[i] > top) top = level[i];
    }
    points_num.assign(top + 1, 0);
    data2file.clear();
    data2file.reserve(n);
    std::vector<std::vector<int> > by_level(top + 1);
    for (unsigned i = 0; i < n; ++i) by_level[level[i]].push_back((int)i);
    for (int l = top; l >= 0; --l) {
        points_num[l] = (int)by_level[l].size();
        data2file.insert(data2file.end(), by_level[l].begin(), by_level[l].end());
    }
}

template <typename T, unsigned A = KGRAPH_MATRIX_ALIGN>
class Matrix {
    unsigned col_ = 0, row_ = 0;
    size_t stride_ = 0;
    char *data_ = nullptr;

    void reset(unsigned r, unsigned c) {
        row_ = r;
        col_ = c;
        stride_ = (sizeof(T) * c + A - 1) / A * A;
        if (data_) free(data_);
        data_ = nullptr;
        void *p = nullptr;
        const size_t bytes = (size_t)r * stride_;
        if (posix_memalign(&p, A, bytes > 0 ? bytes : A) != 0) throw runtime_error("memalign");
        data_ = (char *)p;
    }
    static size_t file_size(std::ifstream &is) {
        is.seekg(0, std::ios::end);
        return (size_t)is.tellg();
    }

public:
    Matrix() {}
    Matrix(unsigned r, unsigned c) { reset(r, c); }
    Matrix(const Matrix &) = delete;
    Matrix &operator=(const Matrix &) = delete;
    ~Matrix() {
        if (data_) free(data_);
    }
    unsigned size() const { return row_; }
    unsigned dim() const { return col_; }
    size_t step() const { return stride_; }
    void resize(unsigned r, unsigned c) { reset(r, c); }
    char *getdata(unsigned i) { return data_ + stride_ * i; }
    T const *operator[](unsigned i) const { return reinterpret_cast<T const *>(data_ + stride_ * i); }
    T *operator[](unsigned i) { return reinterpret_cast<T *>(data_ + stride_ * i); }
    void zero() { memset(data_, 0, (size_t)row_ * stride_); }
    void normalize2() {
        for (unsigned i = 0; i < row_; ++i) {
            T *p = (*this)[i];
            double s = 0;
            for (unsigned j = 0; j < col_; ++j) s += double(p[j]) * double(p[j]);
            s = std::sqrt(s);
            for (unsigned j = 0; j < col_; ++j) p[j] = T(p[j] / s);
        }
    }
    /* raw rows of `dim` values, `skip` header bytes, `gap` bytes after each row */
    void load(const std::string &path, unsigned dim, unsigned skip = 0, unsigned gap = 0) {
        std::ifstream is(path.c_str(), std::ios::binary);
        if (!is) throw io_error(path);
        const size_t line = sizeof(T) * dim + gap;
        const unsigned n = (unsigned)((file_size(is) - skip) / line);
        reset(n, dim);
        zero();
        is.seekg(skip, std::ios::beg);
        for (unsigned i = 0; i < n; ++i) {
            is.read(getdata(i), sizeof(T) * dim);
            is.seekg(gap, std::ios::cur);
        }
        if (!is) throw io_error(path);
    }
    /* lshkit: header {u32 sizeof(T), u32 rows, u32 cols}, then the rows */
    static unsigned lshkit_dim(const std::string &path) {
        std::ifstream is(path.c_str(), std::ios::binary);
        uint32_t h[3];
        is.read((char *)h, sizeof h);
        if (!is || h[0] != sizeof(T)) throw io_error(path);
        return h[2];
    }
    void load_lshkit(const std::string &path) { load(path, lshkit_dim(path), 12, 0); }
    void save_lshkit(const std::string &path) const {
        std::ofstream os(path.c_str(), std::ios::binary);
        const uint32_t h[3] = {(uint32_t)sizeof(T), row_, col_};
        os.write((const char *)h, sizeof h);
        for (unsigned i = 0; i < row_; ++i) os.write(data_ + stride_ * i, sizeof(T) * col_);
        if (!os) throw io_error(path);
    }
    /* rows stored in HNSW level order (highest level first); data2file maps a
     * storage row to its file row; returns the seconds spent on the levels */
    double hnsw_dataload(const std::string &path, unsigned dim, unsigned skip, unsigned gap,
                         std::vector<int> &data2file, std::vector<int> &points_num, unsigned M = 50,
                         unsigned seed = 2024) {
        std::ifstream is(path.c_str(), std::ios::binary);
        if (!is) throw io_error(path);
        const size_t line = sizeof(T) * dim + gap;
        const unsigned n = (unsigned)((file_size(is) - skip) / line);
        std::vector<int> level;
        const double t0 = (double)clock();
        hnsw_levels(n, M, seed, level, data2file, points_num);
        const double secs = ((double)clock() - t0) / CLOCKS_PER_SEC;
        std::vector<int> file2data(n);
        for (unsigned i = 0; i < n; ++i) file2data[data2file[i]] = (int)i;
        reset(n, dim);
        zero();
        is.seekg(skip, std::ios::beg);
        for (unsigned i = 0; i < n; ++i) {
            is.read(getdata(file2data[i]), sizeof(T) * dim);
            is.seekg(gap, std::ios::cur);
        }
        if (!is) throw io_error(path);
        return secs;
    }
};

template <typename MATRIX, typename DIST>
class MatrixOracle : public IndexOracle, public RowSource {
    MATRIX const &m_;
    unsigned size_;
    std::vector<float> selfdot_;

public:
    explicit MatrixOracle(MATRIX const &m) : m_(m), size_(m.size()) {}
    unsigned size() const override { return size_; }
    unsigned data_size() const override { return m_.size(); }
    void set_size(unsigned n) override { size_ = n > m_.size() ? m_.size() : n; } /* src/kgraph-data.h:372-382 */
    unsigned dim() const override { return m_.dim(); }
    float operator()(unsigned i, unsigned j) const override { return DIST::apply(m_[i], m_[j], m_.dim()); }
    float operator()(unsigned i, unsigned j, unsigned off, unsigned d) const override {
        return DIST::apply(m_[i] + off, m_[j] + off, d);
    }
    float operator()(const float *q, unsigned i) const override { return DIST::apply(q, m_[i], m_.dim()); }
    float computeDot(unsigned i, unsigned j) const override { return DIST::dot(m_[i], m_[j], m_.dim()); }
    void computeSelfDotPtr() override {
        selfdot_.resize(m_.size());
        for (unsigned i = 0; i < m_.size(); ++i) selfdot_[i] = DIST::dot(m_[i], m_[i], m_.dim());
    }
    /* mean row, new[]-allocated (caller deletes), src/kgraph-data.h:413-428 */
    float *Calcenter() const override {
        float *c = new float[m_.dim()]();
        for (unsigned i = 0; i < m_.size(); ++i)
            for (unsigned j = 0; j < m_.dim(); ++j) c[j] += m_[i][j];
        for (unsigned j = 0; j < m_.dim(); ++j) c[j] /= m_.size();
        return c;
    }
    const float *rows() const override { return m_[0]; }
    size_t row_stride_bytes() const override { return m_.step(); }

    class Query : public SearchOracle {
        MATRIX const &m_;
        const float *q_;

    public:
        Query(MATRIX const &m, const float *q) : m_(m), q_(q) {}
        unsigned size() const override { return m_.size(); }
        float operator()(unsigned i) const override { return DIST::apply(m_[i], q_, m_.dim()); }
    };
    Query query(const float *q) const { return Query(m_, q); }
};

} // namespace kgraph

#endif
