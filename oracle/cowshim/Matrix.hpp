// Clean-room stand-in for Cow::Matrix (dense row-major FP64 matrix) as used by
// Mara2's ConservationLaw::State and MethodOfLinesWeno.  TEST INFRASTRUCTURE.
#pragma once

#include <stdexcept>
#include <vector>

namespace Cow
{
class Matrix
{
public:
    Matrix() : nr (0), nc (0) {}
    Matrix (int rows, int cols) : nr (rows), nc (cols), D (std::size_t (rows) * cols, 0.0)
    {
        for (int n = 0; n < rows && n < cols; ++n) (*this) (n, n) = 1.0; // identity by default
    }
    double& operator() (int i, int j) { return D[std::size_t (i) * nc + j]; }
    const double& operator() (int i, int j) const { return D[std::size_t (i) * nc + j]; }
    int rows() const { return nr; }
    int cols() const { return nc; }

    Matrix operator* (const Matrix& B) const
    {
        if (nc != B.nr) throw std::logic_error ("Cow shim: matrix shapes do not conform");
        Matrix C;
        C.nr = nr;
        C.nc = B.nc;
        C.D.assign (std::size_t (nr) * B.nc, 0.0);
        for (int i = 0; i < nr; ++i)
            for (int j = 0; j < B.nc; ++j)
            {
                double s = 0.0;
                for (int k = 0; k < nc; ++k) s += (*this) (i, k) * B (k, j);
                C (i, j) = s;
            }
        return C;
    }

private:
    int nr, nc;
    std::vector<double> D;
};
} // namespace Cow
