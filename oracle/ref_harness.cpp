// C-ABI harness around the reference's own CPU sources (compiled in place from
// the read-only reference tree by oracle/build_ref.sh; nothing is copied).
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product links this. It is used to
// generate golden vectors (tests/golden/) and to pin the oracle restatement
// (oracle/freud_oracle.c) against the real reference arithmetic.
//
// Reference entry points driven here:
//   freud/locality/NeighborQuery.h:434-481   NeighborQueryIterator::toNeighborList
//   freud/locality/LinkCell.cc:222-260        LinkCell::LinkCell
//   freud/locality/AABBQuery.cc:18-24         AABBQuery::AABBQuery
//   freud/locality/RawPoints.h:30-77          RawPoints (default (box, points) path)
//   freud/locality/CellQuery.cc:17-137        CellQuery (ghost-particle grid, ball queries)
//   freud/locality/NeighborList.cc:51-82      NeighborList from arrays
//   freud/density/RDF.cc:25-110               RDF ctor / accumulate / reduce
//   freud/density/CorrelationFunction.cc:26-96 CorrelationFunction ctor / accumulate / reduce
//   freud/pmft/PMFTR12.cc, PMFTXYT.cc, PMFTXY.cc, PMFTXYZ.cc   PMFT ctors / accumulate / reduce
//   freud/order/Steinhardt.cc:85-118          Steinhardt::compute
#include <complex>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "AABBQuery.h"
#include "CellQuery.h"
#include "Box.h"
#include "CorrelationFunction.h"
#include "PMFTR12.h"
#include "PMFTXY.h"
#include "PMFTXYT.h"
#include "PMFTXYZ.h"
#include "LinkCell.h"
#include "NeighborList.h"
#include "NeighborQuery.h"
#include "RDF.h"
#include "RawPoints.h"
#include "Steinhardt.h"

using freud::box::Box;
using namespace freud::locality;

namespace {
// Error classes mirror the exception -> Python mapping of the reference bindings.
enum
{
    REF_OK = 0,
    REF_VALUE_ERROR = 1,
    REF_RUNTIME_ERROR = 2,
    REF_INDEX_ERROR = 3,
};

int report(const std::exception& e, int cls, char* err, int errlen)
{
    if (err != nullptr && errlen > 0)
    {
        std::strncpy(err, e.what(), static_cast<size_t>(errlen) - 1);
        err[errlen - 1] = 0;
    }
    return cls;
}

Box make_box(const float* b6, int is2d)
{
    return Box(b6[0], b6[1], b6[2], b6[3], b6[4], b6[5], is2d != 0);
}

std::shared_ptr<NeighborQuery> make_nq(int kind, const Box& box, const float* pts, unsigned n, float cell_width)
{
    const auto* p = reinterpret_cast<const vec3<float>*>(pts);
    if (kind == 0)
    {
        return std::make_shared<RawPoints>(box, p, n);
    }
    if (kind == 3)
    {
        return std::make_shared<CellQuery>(box, p, n);
    }
    if (kind == 1)
    {
        return std::make_shared<AABBQuery>(box, p, n);
    }
    return std::make_shared<LinkCell>(box, p, n, cell_width);
}

QueryArgs make_qargs(int mode, unsigned num_neighbors, float r_max, float r_min, float r_guess, float scale,
                     int exclude_ii)
{
    QueryArgs q;
    q.mode = mode == 1 ? QueryType::ball : (mode == 2 ? QueryType::nearest : QueryType::none);
    q.num_neighbors = num_neighbors;
    q.r_max = r_max;
    q.r_min = r_min;
    q.r_guess = r_guess;
    q.scale = scale;
    q.exclude_ii = exclude_ii != 0;
    return q;
}

struct NlistHandle
{
    std::shared_ptr<NeighborList> nl;
};

std::shared_ptr<NeighborList> nlist_from(unsigned nbonds, const unsigned* ij, unsigned nq, unsigned np,
                                         const float* vec, const float* w)
{
    std::vector<unsigned> qi(nbonds);
    std::vector<unsigned> pi(nbonds);
    for (unsigned b = 0; b < nbonds; ++b)
    {
        qi[b] = ij[2 * b];
        pi[b] = ij[2 * b + 1];
    }
    return std::make_shared<NeighborList>(nbonds, qi.data(), nq, pi.data(), np,
                                          reinterpret_cast<const vec3<float>*>(vec), w);
}
} // namespace

extern "C" {

// kind: 0 = RawPoints (AABB arithmetic), 1 = AABBQuery, 2 = LinkCell(cell_width), 3 = CellQuery
// mode: 0 = infer, 1 = ball, 2 = nearest
void* ref_query(int kind, const float* box6, int is2d, const float* pts, unsigned n, float cell_width,
                const float* qpts, unsigned nq, int mode, unsigned num_neighbors, float r_max, float r_min,
                float r_guess, float scale, int exclude_ii, int sort_by_distance, unsigned* nbonds_out,
                int* status, char* err, int errlen)
{
    *status = REF_OK;
    try
    {
        const Box box = make_box(box6, is2d);
        auto nqo = make_nq(kind, box, pts, n, cell_width);
        auto it = nqo->query(reinterpret_cast<const vec3<float>*>(qpts), nq,
                             make_qargs(mode, num_neighbors, r_max, r_min, r_guess, scale, exclude_ii));
        auto* h = new NlistHandle {it->toNeighborList(sort_by_distance != 0)};
        *nbonds_out = h->nl->getNumBonds();
        return h;
    }
    catch (const std::invalid_argument& e)
    {
        *status = report(e, REF_VALUE_ERROR, err, errlen);
    }
    catch (const std::domain_error& e)
    {
        *status = report(e, REF_VALUE_ERROR, err, errlen);
    }
    catch (const std::out_of_range& e)
    {
        *status = report(e, REF_INDEX_ERROR, err, errlen);
    }
    catch (const std::exception& e)
    {
        *status = report(e, REF_RUNTIME_ERROR, err, errlen);
    }
    return nullptr;
}

void ref_nlist_copy(void* handle, unsigned* ij, float* dist, float* w, float* vec)
{
    auto* h = static_cast<NlistHandle*>(handle);
    const unsigned nb = h->nl->getNumBonds();
    for (unsigned b = 0; b < nb; ++b)
    {
        ij[2 * b] = (*h->nl->getNeighbors())(b, 0);
        ij[2 * b + 1] = (*h->nl->getNeighbors())(b, 1);
        dist[b] = (*h->nl->getDistances())[b];
        w[b] = (*h->nl->getWeights())[b];
        const vec3<float> v = (*h->nl->getVectors())[b];
        vec[3 * b] = v.x;
        vec[3 * b + 1] = v.y;
        vec[3 * b + 2] = v.z;
    }
}

void ref_nlist_free(void* handle)
{
    delete static_cast<NlistHandle*>(handle);
}

// RDF accumulated over nframes (reset=False semantics after the first frame).
// Points of frame f are pts[offsets[f]*3 .. offsets[f+1]*3). When nbonds_per_frame
// is non-null a user NeighborList is given per frame (ij/vec/w concatenated).
int ref_rdf(unsigned bins, float r_max, float r_min, int finite_size, int nframes, const float* boxes6,
            const int* is2d, const unsigned* offsets, const float* pts, int kind, float cell_width, int mode,
            unsigned num_neighbors, float q_r_max, float q_r_min, int exclude_ii,
            const unsigned* nbonds_per_frame, const unsigned* ij, const float* vec, const float* w,
            unsigned* counts, float* rdf, float* nr, char* err, int errlen)
{
    try
    {
        freud::density::RDF r(bins, r_max, r_min);
        if (finite_size != 0)
        {
            r.mode = freud::density::NormalizationMode::finite_size;
        }
        size_t bond_off = 0;
        for (int f = 0; f < nframes; ++f)
        {
            const Box box = make_box(boxes6 + 6 * f, is2d[f]);
            const unsigned n = offsets[f + 1] - offsets[f];
            const float* p = pts + 3 * static_cast<size_t>(offsets[f]);
            auto nqo = make_nq(kind, box, p, n, cell_width);
            std::shared_ptr<NeighborList> nl;
            if (nbonds_per_frame != nullptr)
            {
                nl = nlist_from(nbonds_per_frame[f], ij + 2 * bond_off, n, n, vec + 3 * bond_off, w + bond_off);
                bond_off += nbonds_per_frame[f];
            }
            r.accumulate(nqo, reinterpret_cast<const vec3<float>*>(p), n, nl,
                         make_qargs(mode, num_neighbors, q_r_max, q_r_min, -1.0F, -1.0F, exclude_ii));
        }
        auto c = r.getBinCounts();
        auto g = r.getRDF();
        auto nn = r.getNr();
        for (unsigned i = 0; i < bins; ++i)
        {
            counts[i] = (*c)[i];
            rdf[i] = (*g)[i];
            nr[i] = (*nn)[i];
        }
        return REF_OK;
    }
    catch (const std::invalid_argument& e)
    {
        return report(e, REF_VALUE_ERROR, err, errlen);
    }
    catch (const std::exception& e)
    {
        return report(e, REF_RUNTIME_ERROR, err, errlen);
    }
}

// CorrelationFunction accumulated over nframes (reset=False after the first frame)
// with a live query per frame. values / qvalues: complex double interleaved, per
// point of each frame. qpts == NULL queries each frame's own points (and qvalues
// == NULL uses values). corr: bins complex values interleaved.
int ref_cf(unsigned bins, float r_max, int nframes, const float* boxes6, const int* is2d, const unsigned* offsets,
           const float* pts, const double* values, const unsigned* qoffsets, const float* qpts,
           const double* qvalues, int kind, float cell_width, int mode, unsigned num_neighbors, float q_r_max,
           float q_r_min, int exclude_ii, unsigned* counts, double* corr, char* err, int errlen)
{
    try
    {
        freud::density::CorrelationFunction cf(bins, r_max);
        for (int f = 0; f < nframes; ++f)
        {
            const Box box = make_box(boxes6 + 6 * f, is2d[f]);
            const unsigned n = offsets[f + 1] - offsets[f];
            const float* p = pts + 3 * static_cast<size_t>(offsets[f]);
            const auto* v = reinterpret_cast<const std::complex<double>*>(values) + offsets[f];
            auto nqo = make_nq(kind, box, p, n, cell_width);
            const float* qp = p;
            unsigned nqp = n;
            const std::complex<double>* qv = v;
            if (qpts != nullptr)
            {
                qp = qpts + 3 * static_cast<size_t>(qoffsets[f]);
                nqp = qoffsets[f + 1] - qoffsets[f];
                if (qvalues != nullptr)
                {
                    qv = reinterpret_cast<const std::complex<double>*>(qvalues) + qoffsets[f];
                }
            }
            cf.accumulate(nqo, v, reinterpret_cast<const vec3<float>*>(qp), qv, nqp, nullptr,
                          make_qargs(mode, num_neighbors, q_r_max, q_r_min, -1.0F, -1.0F, exclude_ii));
        }
        auto c = cf.getBinCounts();
        auto g = cf.getCorrelation();
        for (unsigned i = 0; i < bins; ++i)
        {
            counts[i] = (*c)[i];
            corr[2 * i] = (*g)[i].real();
            corr[2 * i + 1] = (*g)[i].imag();
        }
        return REF_OK;
    }
    catch (const std::invalid_argument& e)
    {
        return report(e, REF_VALUE_ERROR, err, errlen);
    }
    catch (const std::exception& e)
    {
        return report(e, REF_RUNTIME_ERROR, err, errlen);
    }
}

// PMFT accumulated over nframes with a live query per frame. kind 0 R12, 1 XYT,
// 2 XY, 3 XYZ. orient: per-point angles (R12, XYT); qorient: per-query angles
// (R12, XYT, XY; NULL: orient) or quaternions (XYZ); qpts == NULL queries the
// frame's points. counts / pcf: row-major over the axes.
int ref_pmft(int kind, const float* maxes, const unsigned* bins, int nframes, const float* boxes6, const int* is2d,
             const unsigned* offsets, const float* pts, const float* orient, const unsigned* qoffsets,
             const float* qpts, const float* qorient, const float* equiv, unsigned n_equiv, int nq_kind, int mode,
             unsigned num_neighbors, float q_r_max, float q_r_min, int exclude_ii, unsigned* counts, float* pcf,
             char* err, int errlen)
{
    try
    {
        std::unique_ptr<freud::pmft::PMFT> pm;
        freud::pmft::PMFTR12* r12 = nullptr;
        freud::pmft::PMFTXYT* xyt = nullptr;
        freud::pmft::PMFTXY* xy = nullptr;
        freud::pmft::PMFTXYZ* xyz = nullptr;
        if (kind == 0)
            pm.reset(r12 = new freud::pmft::PMFTR12(maxes[0], bins[0], bins[1], bins[2]));
        else if (kind == 1)
            pm.reset(xyt = new freud::pmft::PMFTXYT(maxes[0], maxes[1], bins[0], bins[1], bins[2]));
        else if (kind == 2)
            pm.reset(xy = new freud::pmft::PMFTXY(maxes[0], maxes[1], bins[0], bins[1]));
        else
            pm.reset(xyz = new freud::pmft::PMFTXYZ(maxes[0], maxes[1], maxes[2], bins[0], bins[1], bins[2]));
        for (int f = 0; f < nframes; ++f)
        {
            const Box box = make_box(boxes6 + 6 * f, is2d[f]);
            const unsigned n = offsets[f + 1] - offsets[f];
            const float* p = pts + 3 * static_cast<size_t>(offsets[f]);
            auto nqo = make_nq(nq_kind, box, p, n, 0.0F);
            const float* qp = p;
            unsigned nqp = n;
            size_t qbase = offsets[f];
            if (qpts != nullptr)
            {
                qp = qpts + 3 * static_cast<size_t>(qoffsets[f]);
                nqp = qoffsets[f + 1] - qoffsets[f];
                qbase = qoffsets[f];
            }
            const auto qargs = make_qargs(mode, num_neighbors, q_r_max, q_r_min, -1.0F, -1.0F, exclude_ii);
            const auto* qv = reinterpret_cast<const vec3<float>*>(qp);
            if (r12 != nullptr || xyt != nullptr)
            {
                const float* o = orient + offsets[f];
                const float* qo = qorient != nullptr ? qorient + qbase : o;
                if (r12 != nullptr)
                    r12->accumulate(nqo, o, qv, qo, nqp, nullptr, qargs);
                else
                    xyt->accumulate(nqo, o, qv, qo, nqp, nullptr, qargs);
            }
            else if (xy != nullptr)
            {
                xy->accumulate(nqo, qorient + qbase, qv, nqp, nullptr, qargs);
            }
            else
            {
                xyz->accumulate(nqo, reinterpret_cast<const quat<float>*>(qorient) + qbase, qv, nqp,
                                reinterpret_cast<const quat<float>*>(equiv), n_equiv, nullptr, qargs);
            }
        }
        auto c = pm->getBinCounts();
        auto g = pm->getPCF();
        for (size_t i = 0; i < c->size(); ++i)
        {
            counts[i] = (*c)[i];
            pcf[i] = (*g)[i];
        }
        return REF_OK;
    }
    catch (const std::invalid_argument& e)
    {
        return report(e, REF_VALUE_ERROR, err, errlen);
    }
    catch (const std::exception& e)
    {
        return report(e, REF_RUNTIME_ERROR, err, errlen);
    }
}

// Steinhardt on one frame. qlm_out holds, per particle, the concatenation over ls of
// the 2l+1 complex values (interleaved re/im floats). Outputs may be null when the
// corresponding option is off.
int ref_steinhardt(const unsigned* ls, unsigned nl, int average, int wl, int weighted, int wl_normalize,
                   const float* box6, int is2d, const float* pts, unsigned n, int kind, float cell_width,
                   int mode, unsigned num_neighbors, float q_r_max, float q_r_min, int exclude_ii,
                   int use_nlist, unsigned nbonds, const unsigned* ij, const float* vec, const float* w,
                   float* ql_out, float* particle_order_out, float* qlm_out, float* order_out, char* err,
                   int errlen)
{
    try
    {
        std::vector<unsigned> lv(ls, ls + nl);
        freud::order::Steinhardt st(lv, average != 0, wl != 0, weighted != 0, wl_normalize != 0);
        const Box box = make_box(box6, is2d);
        auto nqo = make_nq(kind, box, pts, n, cell_width);
        std::shared_ptr<NeighborList> nlist;
        if (use_nlist != 0)
        {
            nlist = nlist_from(nbonds, ij, n, n, vec, w);
        }
        st.compute(nlist, nqo, make_qargs(mode, num_neighbors, q_r_max, q_r_min, -1.0F, -1.0F, exclude_ii));
        auto ql = st.getQl();
        auto po = st.getParticleOrder();
        for (size_t i = 0; i < static_cast<size_t>(n) * nl; ++i)
        {
            ql_out[i] = ql->data()[i];
            particle_order_out[i] = po->data()[i];
        }
        const auto& qlm = st.getQlm();
        size_t stride = 0;
        for (unsigned k = 0; k < nl; ++k)
        {
            stride += 2 * lv[k] + 1;
        }
        size_t off = 0;
        for (unsigned k = 0; k < nl; ++k)
        {
            const size_t nm = 2 * lv[k] + 1;
            for (size_t i = 0; i < n; ++i)
            {
                for (size_t m = 0; m < nm; ++m)
                {
                    const std::complex<float> v = qlm[k]->data()[i * nm + m];
                    qlm_out[2 * (i * stride + off + m)] = v.real();
                    qlm_out[2 * (i * stride + off + m) + 1] = v.imag();
                }
            }
            off += nm;
        }
        auto order = st.getOrder();
        for (unsigned k = 0; k < nl; ++k)
        {
            order_out[k] = order[k];
        }
        return REF_OK;
    }
    catch (const std::invalid_argument& e)
    {
        return report(e, REF_VALUE_ERROR, err, errlen);
    }
    catch (const std::exception& e)
    {
        return report(e, REF_RUNTIME_ERROR, err, errlen);
    }
}

} // extern "C"
