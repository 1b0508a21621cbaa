// mini_grid.hpp -- test stand-in for MMSP's grid container (tests only).
//
// It offers the subset of MMSP::grid / MMSP::vector that MMSP.gpu.hpp uses
// (include/MMSP.grid.h:263-337 free functions, operator()(int) of
// include/MMSP.grid.cpp:385-400, vector<T>::operator[]) with the same
// semantics for a serial, periodic grid, so the drop-in wrapper can be run on
// a machine that does not hold the reference headers.
#ifndef MINI_GRID_HPP
#define MINI_GRID_HPP
#include <cstdarg>
#include <cstdlib>
#include <utility>
#include <vector>

namespace MMSP {

inline void Abort(int err) { std::exit(err); }

template <typename T> class vector {
public:
    vector() {}
    explicit vector(int n, T v = T()) : d(n, v) {}
    T& operator[](int i) { return d[i]; }
    const T& operator[](int i) const { return d[i]; }
    int length() const { return (int)d.size(); }
    void resize(int n) { d.resize(n); }
private:
    std::vector<T> d;
};

// the sparse cell of include/MMSP.sparse.h:19: (index, value) items in
// insertion order; set() overwrites an item or appends one
template <typename T> class sparse {
public:
    T& set(int index)
    {
        for (size_t h = 0; h < d.size(); h++)
            if (d[h].first == index) return d[h].second;
        d.push_back(std::make_pair(index, T(0)));
        return d.back().second;
    }
    int length() const { return (int)d.size(); }
    int index(int h) const { return d[h].first; }
    T value(int h) const { return d[h].second; }
private:
    std::vector<std::pair<int, T> > d;
};
template <typename T> int length(const sparse<T>& s) { return s.length(); }
template <typename T> T& set(sparse<T>& s, int index) { return s.set(index); }
template <typename T> int index(const sparse<T>& s, int h) { return s.index(h); }
template <typename T> T value(const sparse<T>& s, int h) { return s.value(h); }

template <typename T> inline void resize_cell(T&, int) {}
template <typename T> inline void resize_cell(vector<T>& v, int n) { v.resize(n); }

template <int dim, typename T> class grid {
public:
    // grid(fields, g0[0], g1[0], g0[1], g1[1], ...) as include/MMSP.grid.cpp:44-69
    grid(int FIELDS, ...) : nf(FIELDS), nn(1)
    {
        va_list l;
        va_start(l, FIELDS);
        for (int i = 0; i < dim; i++) {
            lo[i] = va_arg(l, int);
            hi[i] = va_arg(l, int);
            nn *= hi[i] - lo[i];
            bc0[i] = bc1[i] = 2;
            h[i] = 1.0;
        }
        va_end(l);
        cells.resize(nn);
        for (int i = 0; i < nn; i++) resize_cell(cells[i], nf);
    }
    T& operator()(int i) const { return const_cast<T&>(cells[i]); }
    friend int nodes(const grid& g) { return g.nn; }
    friend int fields(const grid& g) { return g.nf; }
    friend int g0(const grid& g, int i) { return g.lo[i]; }
    friend int g1(const grid& g, int i) { return g.hi[i]; }
    friend int x0(const grid& g, int i) { return g.lo[i]; }
    friend int x1(const grid& g, int i) { return g.hi[i]; }
    friend int b0(const grid& g, int i) { return g.bc0[i]; }
    friend int b1(const grid& g, int i) { return g.bc1[i]; }
    friend int& b0(grid& g, int i) { return g.bc0[i]; }
    friend int& b1(grid& g, int i) { return g.bc1[i]; }
    friend double dx(const grid& g, int i) { return g.h[i]; }
    friend double& dx(grid& g, int i) { return g.h[i]; }
private:
    int nf, nn;
    int lo[dim], hi[dim], bc0[dim], bc1[dim];
    double h[dim];
    std::vector<T> cells;
};

}  // namespace MMSP
#endif
