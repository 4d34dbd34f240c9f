// Stand-in for the fsph header that the reference's Steinhardt.cc includes
// (the fsph submodule is not vendored). Test infrastructure only: it exists so
// the reference CPU sources compile into a golden-vector generator.
//
// Contract, pinned by the reference's own test_qlmi (values compared against
// scipy.special.sph_harm_y after Steinhardt.cc applies (-1)^m to positive odd m):
// compute(polar, azimuth) stores, for every l <= max_l, the 2l+1 values
// N_l^|m| P_l^|m|(cos polar) exp(i m azimuth) in the order m = 0..l, -1..-l,
// where P has no Condon-Shortley phase and N = sqrt((2l+1)/(4 pi) (l-|m|)!/(l+|m|)!).
// Evaluated in double and rounded to Real.
#ifndef FG_FSPH_STANDIN_HPP
#define FG_FSPH_STANDIN_HPP
#include <cmath>
#include <complex>
#include <vector>

namespace fsph {
template<typename Real> class PointSPHEvaluator
{
public:
    using iterator = typename std::vector<std::complex<Real>>::const_iterator;

    explicit PointSPHEvaluator(unsigned int max_l) : m_max_l(max_l), m_values((max_l + 2) * (max_l + 2)) {}

    // First argument: polar angle; second: azimuthal angle.
    void compute(Real polar, Real azimuth)
    {
        const int L = static_cast<int>(m_max_l);
        const double x = std::cos(static_cast<double>(polar));
        const double s = std::sqrt(std::max(0.0, 1.0 - x * x));
        const double az = static_cast<double>(azimuth);
        std::vector<double> p((L + 1) * (L + 1), 0.0); // p[l*(L+1)+m], unnormalised, no CS phase
        double pmm = 1.0;
        for (int m = 0; m <= L; ++m)
        {
            if (m > 0)
            {
                pmm *= (2.0 * m - 1.0) * s;
            }
            p[m * (L + 1) + m] = pmm;
            if (m + 1 <= L)
            {
                p[(m + 1) * (L + 1) + m] = x * (2.0 * m + 1.0) * pmm;
            }
            for (int l = m + 2; l <= L; ++l)
            {
                p[l * (L + 1) + m] = ((2.0 * l - 1.0) * x * p[(l - 1) * (L + 1) + m]
                                      - (l + m - 1.0) * p[(l - 2) * (L + 1) + m])
                    / (l - m);
            }
        }
        for (int l = 0; l <= L; ++l)
        {
            const std::size_t base = static_cast<std::size_t>(l) * static_cast<std::size_t>(l);
            for (int m = 0; m <= l; ++m)
            {
                double ratio = 1.0; // (l-m)!/(l+m)!
                for (int k = l - m + 1; k <= l + m; ++k)
                {
                    ratio /= k;
                }
                const double norm = std::sqrt((2.0 * l + 1.0) / (4.0 * M_PI) * ratio) * p[l * (L + 1) + m];
                const double c = norm * std::cos(m * az);
                const double sn = norm * std::sin(m * az);
                m_values[base + m] = std::complex<Real>(static_cast<Real>(c), static_cast<Real>(sn));
                if (m > 0)
                {
                    m_values[base + l + m] = std::complex<Real>(static_cast<Real>(c), static_cast<Real>(-sn));
                }
            }
        }
    }

    // Iterator to the value block of degree l (m order 0..l, -1..-l). Only m = 0
    // and full = true are used by the callers.
    iterator begin_l(unsigned int l, unsigned int /*m*/, bool /*full*/) const
    {
        return m_values.begin() + static_cast<std::ptrdiff_t>(l) * static_cast<std::ptrdiff_t>(l);
    }

private:
    unsigned int m_max_l;
    std::vector<std::complex<Real>> m_values;
};
}; // namespace fsph
#endif
