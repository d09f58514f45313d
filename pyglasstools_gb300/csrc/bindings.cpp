// bindings.cpp -- pybind11 modules with the reference's class and method names
// (_pyglasstools, _potential, _cgfunc, _irvingkirkwood), thin over the C ABI of
// libik_gb300.so (include/ik_gb300.h).  Every numeric evaluation goes to the GPU.
//
// Mirrors: module-pyglasstools.cpp, ParticleSystem.cc:199-221, SimBox.cc:55-69,
// potential/PairPotential.h:125-152, irvingkirkwood/cgfunc/CoarseGrainFunction.h:136-167,
// irvingkirkwood/IrvingKirkwood.h:113-122, irvingkirkwood/CoarseGrainedField.h:342-358.
#include <pybind11/numpy.h>
#include <charconv>
#include <cstdio>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ik_gb300.h"

namespace py = pybind11;
using Vec3 = std::array<double, 3>;
using DArr = py::array_t<double, py::array::c_style | py::array::forcecast>;

static void check(int rc)
{
    if (rc != IK_OK) {
        std::string msg = ik_last_error();
        if (rc == IK_ERR_ARG || rc == IK_ERR_BOX) throw std::invalid_argument("[ERROR]: " + msg);
        throw std::runtime_error("[ERROR]: " + msg);
    }
}

// One shared context for scalar evaluations (getPairForceDivR, getBondFunc, ...).
static ik_ctx* util_ctx()
{
    static ik_ctx* c = nullptr;
    static std::mutex m;
    std::lock_guard<std::mutex> lk(m);
    if (!c) check(ik_create(&c, 0));
    return c;
}

static std::vector<double> to_xyz(py::handle obj, size_t expect_rows, const char* what)
{
    DArr a = DArr::ensure(obj);
    if (!a) throw std::invalid_argument(std::string("[ERROR]: ") + what + " must be array-like");
    auto b = a.request();
    std::vector<double> out;
    size_t rows = b.ndim >= 1 ? (size_t)b.shape[0] : 0;
    size_t cols = b.ndim == 2 ? (size_t)b.shape[1] : (b.ndim == 1 ? 1 : 0);
    if (b.ndim == 1 && expect_rows == 1) { rows = 1; cols = (size_t)b.shape[0]; }
    if (b.ndim > 2 || cols < 2 || cols > 3)
        throw std::invalid_argument(std::string("[ERROR]: ") + what + " must be (n, 2) or (n, 3)");
    if (expect_rows != (size_t)-1 && rows != expect_rows)
        throw std::invalid_argument(std::string("[ERROR]: Size of ") + what + " array mismatch with # of particles!");
    out.assign(rows * 3, 0.0);
    const double* p = static_cast<const double*>(b.ptr);
    for (size_t i = 0; i < rows; ++i)
        for (size_t c = 0; c < cols; ++c) out[3 * i + c] = p[i * cols + c];
    return out;
}

static std::vector<double> to_vec(py::handle obj, const char* what)
{
    DArr a = DArr::ensure(obj);
    if (!a) throw std::invalid_argument(std::string("[ERROR]: ") + what + " must be array-like");
    auto b = a.request();
    const double* p = static_cast<const double*>(b.ptr);
    return std::vector<double>(p, p + b.size);
}

static Vec3 to3(py::handle obj)
{
    std::vector<double> v = to_vec(obj, "vector");
    Vec3 r = {0, 0, 0};
    for (size_t k = 0; k < v.size() && k < 3; ++k) r[k] = v[k];
    return r;
}

// ---------------------------------------------------------------- _pyglasstools
struct SimBox {
    int dim = 3;
    Vec3 origin{}, boxsize{}, lowerbound{}, upperbound{}, periodic{};
    double vol = 0.0;
    SimBox(Vec3 L, Vec3 o, int d) { init(L, o, d); }
    void init(Vec3 L, Vec3 o, int d)
    {
        // SimBox.cc:25-52 (bounds set before the 2D z overrides, as in the reference)
        dim = d;
        origin = o;
        boxsize = L;
        for (int a = 0; a < 3; ++a) {
            upperbound[a] = 0.5 * boxsize[a] - origin[a];
            lowerbound[a] = -upperbound[a] - 2.0 * origin[a];
            periodic[a] = 1;
        }
        if (dim == 2) {
            boxsize[2] = 1.0;
            periodic[2] = 0;
            origin[2] = 0.0;
            vol = boxsize[0] * boxsize[1];
        } else {
            vol = boxsize[0] * boxsize[1] * boxsize[2];
        }
    }
    Vec3 minImage(Vec3 v) const
    {
        Vec3 w = v;
        for (int a = 2; a >= 0; --a)
            if (periodic[a]) w[a] -= boxsize[a] * (double)rintf((float)(w[a] / boxsize[a]));
        return w;
    }
};

struct ParticleSystem {
    std::shared_ptr<SimBox> simbox;
    unsigned int N = 0;
    std::vector<double> diameter, mass, pos, vel, disp;
    uint64_t version = 0;
    ik_ctx* qctx = nullptr;      // lazily created context for neighbour queries
    uint64_t qversion = (uint64_t)-1;

    ParticleSystem(std::shared_ptr<SimBox> box, unsigned int n, py::handle d, py::handle m, py::handle p,
                   py::handle v)
        : simbox(std::move(box))
    {
        set(n, d, m, p, v);
    }
    ~ParticleSystem() { if (qctx) ik_destroy(qctx); }
    void set(unsigned int n, py::handle d, py::handle m, py::handle p, py::handle v)
    {
        N = n;
        diameter = to_vec(d, "diameter");
        mass = to_vec(m, "mass");
        if (diameter.size() != n) throw std::invalid_argument("[ERROR]: Size of diameter array mismatch with # of particles!");
        if (mass.size() != n) throw std::invalid_argument("[ERROR]: Size of mass array mismatch with # of particles!");
        pos = to_xyz(p, n, "position");
        vel = to_xyz(v, n, "velocity");
        disp.assign(3 * (size_t)n, 0.0);
        ++version;
    }
    ik_ctx* query_ctx()
    {
        if (!qctx) check(ik_create(&qctx, 0));
        if (qversion != version) {
            double L[3] = {simbox->boxsize[0], simbox->boxsize[1], simbox->boxsize[2]};
            double o[3] = {simbox->origin[0], simbox->origin[1], simbox->origin[2]};
            check(ik_set_box(qctx, simbox->dim, L, o));
            check(ik_set_frame(qctx, N, pos.data(), vel.data(), mass.data(), diameter.data()));
            check(ik_synchronize(qctx));
            qversion = version;
        }
        return qctx;
    }
    std::vector<unsigned int> getNeighbors(py::handle point, double radius)
    {
        Vec3 q = to3(point);
        ik_ctx* c = query_ctx();
        int64_t cnt = 0;
        check(ik_get_neighbors_point(c, 0, q.data(), radius, nullptr, 0, &cnt));
        std::vector<int32_t> ids((size_t)std::max<int64_t>(cnt, 1));
        check(ik_get_neighbors_point(c, 0, q.data(), radius, ids.data(), cnt, &cnt));
        return std::vector<unsigned int>(ids.begin(), ids.begin() + cnt);
    }
    py::array_t<double> getNeighborsDistance(int tag, double radius)
    {
        if (tag < 0 || (unsigned)tag >= N) throw std::invalid_argument("[ERROR]: particle tag out of range");
        ik_ctx* c = query_ctx();
        std::vector<int64_t> offs(N + 1);
        int64_t nnz = 0;
        check(ik_get_neighbors(c, 0, radius, offs.data(), nullptr, 0, &nnz));
        std::vector<int32_t> idx((size_t)std::max<int64_t>(nnz, 1));
        check(ik_get_neighbors(c, 0, radius, offs.data(), idx.data(), nnz, &nnz));
        int64_t s = offs[(size_t)tag], e = offs[(size_t)tag + 1];
        py::array_t<double> out({(py::ssize_t)(e - s), (py::ssize_t)3});
        auto o = out.mutable_unchecked<2>();
        for (int64_t k = s; k < e; ++k) {
            int j = idx[(size_t)k];
            for (int a = 0; a < 3; ++a) {
                double d = pos[3 * (size_t)j + a] - pos[3 * (size_t)tag + a];
                if (simbox->periodic[a]) d = d - simbox->boxsize[a] * std::nearbyint(d / simbox->boxsize[a]);
                o(k - s, a) = d;
            }
        }
        return out;
    }
    py::tuple neighborList(double radius)
    {
        ik_ctx* c = query_ctx();
        py::array_t<int64_t> offs((py::ssize_t)N + 1);
        int64_t nnz = 0;
        check(ik_get_neighbors(c, 0, radius, offs.mutable_data(), nullptr, 0, &nnz));
        py::array_t<int32_t> idx((py::ssize_t)nnz);
        check(ik_get_neighbors(c, 0, radius, offs.mutable_data(), idx.mutable_data(), nnz, &nnz));
        return py::make_tuple(offs, idx);
    }
    static py::array_t<double> as_nx3(const std::vector<double>& v)
    {
        py::array_t<double> a({(py::ssize_t)(v.size() / 3), (py::ssize_t)3});
        std::copy(v.begin(), v.end(), a.mutable_data());
        return a;
    }
};

// Single-rank communicator with the methods the Python layer uses (MPIInterface.h:58-441).
struct Communicator {
    int getRank() const { return 0; }
    int getSizeGlobal() const { return 1; }
    void barrier() const {}
    void abort(int code) const { std::fflush(nullptr); std::_Exit(code); }
    py::object bcast(py::object v, int) const { return v; }
    py::object scatter_v(py::list parts, int) const { return parts.size() ? parts[0] : py::object(py::none()); }
    py::object gather_v(py::object v, int) const { py::list l; l.append(v); return std::move(l); }
    py::object all_gather_v(py::object v) const { py::list l; l.append(v); return std::move(l); }
    void send(py::object, int, int) const {}
    py::object recv(int, int) const { return py::bool_(true); }
};

// Buffered stand-in of MPI::LogFile (MPIFile.h:23-56): write_shared appends.
struct MPILogFile {
    std::ofstream f;
    MPILogFile(std::shared_ptr<Communicator>, const std::string& name) : f(name, std::ios::out | std::ios::app)
    {
        if (!f) throw std::runtime_error("[ERROR]: cannot open " + name);
    }
    void write_shared(const std::string& s) { f << s; }
    void flush() { f.flush(); }
    void close() { f.close(); }
};

struct Manager {
    int notice_level = 2;
};

// ---------------------------------------------------------------- _potential
struct PairPotential {
    double scaled_rcut = 0.0;
    std::vector<double> params;
    PairPotential(std::vector<double> p) : params(std::move(p)) {}
    PairPotential(double rc, std::vector<double> p) : scaled_rcut(rc), params(std::move(p)) {}
    virtual ~PairPotential() = default;
    virtual int model() const { return -1; }
    virtual double getRcut(py::handle, double, double) { return 0.0; }
    virtual double getPairForceDivR(py::handle, double, double) { return 0.0; }
    virtual double getPairEnergy(py::handle, double, double) { return 0.0; }
    void setParams(double v, int k)
    {
        if (k < 0 || (size_t)k >= params.size()) throw std::invalid_argument("[ERROR]: parameter index out of range");
        params[(size_t)k] = v;
    }
    std::vector<double> getParams() const { return params; }
};

// ShortRangePairPotential<Model> for the eight models (potential/PairPotential.h:69-123,
// potential/module-potential.cpp:13-34); the force and energy are evaluated on the
// device (ik_eval_pair), getRcut on the host as Model::computeRcut.
template <int KIND>
struct ShortRangePairPotential : PairPotential {
    using PairPotential::PairPotential;
    int model() const override { return KIND; }
    void validate() const
    {
        const int need = ik_potential_nparams(KIND);
        if ((int)params.size() < need)
            throw std::invalid_argument("[ERROR]: this pair potential needs " + std::to_string(need) +
                                        " parameters, got " + std::to_string(params.size()));
    }
    // computeRcut: rcutsq sigma^2 with the non-additive sigma (the force-shifted LJ
    // inherits LennardJones::computeRcut, LennardJones.h:77-81)
    double getRcut(py::handle, double di, double dj) override
    {
        validate();
        const double eps = KIND == IK_POT_POLYYUKAWA ? params[2] : params[1];
        const double s = 0.5 * (di + dj) * (1 - eps * std::fabs(di - dj));
        return scaled_rcut * scaled_rcut * s * s;
    }
    std::pair<double, double> eval(py::handle rij, double di, double dj)
    {
        validate();
        Vec3 r = to3(rij);
        ik_ctx* c = util_ctx();
        check(ik_set_potential(c, KIND, scaled_rcut, params.data(), (int)params.size()));
        double f = 0, e = 0;
        check(ik_eval_pair(c, 1, r.data(), &di, &dj, &f, &e));
        return {f, e};
    }
    double getPairForceDivR(py::handle rij, double di, double dj) override { return eval(rij, di, dj).first; }
    double getPairEnergy(py::handle rij, double di, double dj) override { return eval(rij, di, dj).second; }
};
using PairPotentialPoly12 = ShortRangePairPotential<IK_POT_POLY12>;

// ---------------------------------------------------------------- _cgfunc
struct CoarseGrainFunction {
    int kind = 0, mode = IK_QUAD_FIXEDPOINT, order = 1, neval = 1000;
    double cg_rcut = 0.0, width = 0.0, relerr = 1e-9, abserr = 1e-9;
    CoarseGrainFunction(double rc) : cg_rcut(rc) {}
    virtual ~CoarseGrainFunction() = default;
    void setRcut(double rc) { cg_rcut = rc; }
    double getRcut() const { return cg_rcut; }
    void apply(ik_ctx* c) const
    {
        check(ik_set_cgfunc(c, kind, mode, order, cg_rcut, width));
        if (mode == IK_QUAD_ADAPTIVE) check(ik_set_adaptive(c, neval, relerr, abserr));
    }
    std::pair<double, double> eval(py::handle x, py::handle ri, py::handle rij) const
    {
        Vec3 a = to3(x), b = to3(ri), r = to3(rij);
        ik_ctx* c = util_ctx();
        apply(c);
        double bond = 0, delta = 0;
        check(ik_eval_bond(c, 1, a.data(), b.data(), r.data(), &bond, &delta));
        return {bond, delta};
    }
    double getDeltaFunc(py::handle x, py::handle ri) const
    {
        return eval(x, ri, py::cast(std::vector<double>{0.0, 0.0, 0.0})).second;
    }
    double getObjFunc(double s, py::handle x, py::handle ri, py::handle rij) const
    {
        Vec3 b = to3(ri), r = to3(rij);
        std::vector<double> p = {b[0] + s * r[0], b[1] + s * r[1], b[2] + s * r[2]};
        return getDeltaFunc(x, py::cast(p));
    }
    double getBondFunc(py::handle x, py::handle ri, py::handle rij) const { return eval(x, ri, rij).first; }
};

template <int KIND>
struct CGFixed : CoarseGrainFunction {
    CGFixed(int ord, double rc) : CoarseGrainFunction(rc)
    {
        kind = KIND;
        mode = IK_QUAD_FIXEDPOINT;
        order = ord;
        if (KIND == IK_CG_MOLLIFIER) width = rc; // normalisation radius frozen at construction
    }
};
template <int KIND>
struct CGAdaptive : CoarseGrainFunction {
    CGAdaptive(int nev, double rel, double abs_, double rc) : CoarseGrainFunction(rc)
    {
        kind = KIND;
        mode = IK_QUAD_ADAPTIVE;
        neval = nev;
        relerr = rel;
        abserr = abs_;
        if (KIND == IK_CG_MOLLIFIER) width = rc;
    }
};
// Gaussian: support R = cut * width (new kernel, not in the reference)
struct CGGaussianFixed : CoarseGrainFunction {
    CGGaussianFixed(int ord, double w, double cut) : CoarseGrainFunction(cut * w)
    {
        kind = IK_CG_GAUSSIAN;
        mode = IK_QUAD_FIXEDPOINT;
        order = ord;
        width = w;
    }
};

struct CGGaussianAdaptive : CoarseGrainFunction {
    CGGaussianAdaptive(int nev, double rel, double abs_, double w, double cut) : CoarseGrainFunction(cut * w)
    {
        kind = IK_CG_GAUSSIAN;
        mode = IK_QUAD_ADAPTIVE;
        neval = nev;
        relerr = rel;
        abserr = abs_;
        width = w;
    }
};

// ---------------------------------------------------------------- text output
// Python's repr() of a float (the "{} ".format(x) of fieldlogger.save_perrank,
// io.py:112-128): the shortest digits that round-trip, fixed notation for decimal
// exponents in [-4, 16) with ".0" on integral values, else d.ddde+XX.
static void py_float_repr(double v, std::string& out)
{
    if (std::isnan(v)) { out += "nan"; return; }
    if (std::isinf(v)) { out += v > 0 ? "inf" : "-inf"; return; }
    if (v == 0.0) { out += std::signbit(v) ? "-0.0" : "0.0"; return; }
    char buf[64];
    auto res = std::to_chars(buf, buf + sizeof buf, v, std::chars_format::scientific);
    std::string sci(buf, res.ptr);          // [-]d[.ddd]e[+-]XX
    const bool neg = sci[0] == '-';
    if (neg) sci.erase(0, 1);
    const size_t epos = sci.find('e');
    const int e10 = std::atoi(sci.c_str() + epos + 1);
    std::string digits;
    for (size_t k = 0; k < epos; ++k) if (sci[k] != '.') digits += sci[k];
    while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
    if (neg) out += '-';
    if (e10 >= -4 && e10 < 16) {
        const int point = e10 + 1; // digits before the decimal point
        if (point <= 0) {
            out += "0.";
            out.append((size_t)(-point), '0');
            out += digits;
        } else if ((size_t)point >= digits.size()) {
            out += digits;
            out.append((size_t)point - digits.size(), '0');
            out += ".0";
        } else {
            out += digits.substr(0, (size_t)point);
            out += '.';
            out += digits.substr((size_t)point);
        }
    } else {
        out += digits[0];
        if (digits.size() > 1) { out += '.'; out += digits.substr(1); }
        char eb[16];
        std::snprintf(eb, sizeof eb, "e%c%02d", e10 < 0 ? '-' : '+', e10 < 0 ? -e10 : e10);
        out += eb;
    }
}

// ---------------------------------------------------------------- _irvingkirkwood
struct CoarseGrainedField {
    std::string name, type;
    bool islocal = false;
    int dim = 2;
    int field = IK_FIELD_VIRIAL;
    std::vector<double> val; // gridsize x dim x dim, column-major per grid point
    py::object gridpoints = py::none();
    CoarseGrainedField(std::string n, std::string t, bool local, int gridsize, int d, int f)
        : name(std::move(n)), type(std::move(t)), islocal(local), dim(d), field(f)
    {
        if (gridsize < 0) throw std::invalid_argument("[ERROR]: gridsize must be >= 0");
        val.assign((size_t)gridsize * d * d, 0.0);
    }
    virtual ~CoarseGrainedField() = default;
    void addGridpoints(py::object g) { gridpoints = std::move(g); }
    std::string gettostring(int index, int grid_id) const
    {
        // CoarseGrainedField.h:284-307: default ostream formatting (6 significant digits) + " "
        size_t DD = (size_t)dim * dim;
        if (grid_id < 0 || (size_t)grid_id * DD >= val.size() || index < 0 || (size_t)index >= DD)
            throw std::out_of_range("[ERROR]: grid/component index out of range");
        std::ostringstream os;
        os << val[(size_t)grid_id * DD + (size_t)index] << " ";
        return os.str();
    }
    void save(MPILogFile& f, int index, int grid_id) { f.write_shared(gettostring(index, grid_id)); }
    void clear(int grid_id)
    {
        size_t DD = (size_t)dim * dim;
        if (grid_id < 0 || (size_t)grid_id * DD >= val.size()) throw std::out_of_range("[ERROR]: grid index out of range");
        std::fill(val.begin() + (long)grid_id * DD, val.begin() + (long)(grid_id + 1) * DD, 0.0);
    }
    py::array_t<double> values() const
    {
        size_t G = val.size() / ((size_t)dim * dim);
        py::array_t<double> a({(py::ssize_t)G, (py::ssize_t)dim, (py::ssize_t)dim});
        auto m = a.mutable_unchecked<3>();
        for (size_t g = 0; g < G; ++g)
            for (int i = 0; i < dim; ++i)
                for (int j = 0; j < dim; ++j) m(g, i, j) = val[g * dim * dim + i + dim * j];
        return a;
    }
};

template <int D, int FIELD>
struct FieldT : CoarseGrainedField {
    FieldT(std::string n, std::string t, bool local, int gridsize)
        : CoarseGrainedField(std::move(n), std::move(t), local, gridsize, D, FIELD)
    {
    }
};

struct IrvingKirkwood {
    std::shared_ptr<ParticleSystem> sys;
    std::shared_ptr<PairPotential> pot;
    std::shared_ptr<CoarseGrainFunction> cg;
    std::shared_ptr<Communicator> comm;
    std::map<std::string, std::shared_ptr<CoarseGrainedField>> obs;
    ik_ctx* ctx = nullptr;
    double max_rcut = 0.0;
    int precision = IK_PREC_FP32;
    uint64_t uploaded = (uint64_t)-1;
    const ParticleSystem* uploaded_sys = nullptr;
    std::vector<double> last_grid;

    IrvingKirkwood(std::shared_ptr<ParticleSystem> s, std::shared_ptr<PairPotential> p,
                   std::shared_ptr<CoarseGrainFunction> c, std::shared_ptr<Communicator> cm)
        : sys(std::move(s)), pot(std::move(p)), cg(std::move(c)), comm(std::move(cm))
    {
        if (!sys || !pot || !cg) throw std::invalid_argument("[ERROR]: IrvingKirkwood needs sysdata, potential, cgfunc");
        // Calculator.h:41-45: frozen at construction
        double dmax = 0.0;
        for (double d : sys->diameter) dmax = std::max(dmax, d);
        max_rcut = std::max(pot->scaled_rcut * dmax, dmax);
        check(ik_create(&ctx, 0));
    }
    ~IrvingKirkwood() { if (ctx) ik_destroy(ctx); }
    void setSystemData(std::shared_ptr<ParticleSystem> s) { sys = std::move(s); }
    void addObservable(std::shared_ptr<CoarseGrainedField> f) { obs[f->name] = std::move(f); }
    void printDisplacement()
    {
        for (unsigned i = 0; i < sys->N; ++i) py::print(sys->disp[3 * i], sys->disp[3 * i + 1], i);
    }
    void setPrecision(const std::string& p)
    {
        if (p == "fp64") precision = IK_PREC_FP64;
        else if (p == "fp32") precision = IK_PREC_FP32;
        else throw std::invalid_argument("[ERROR]: precision must be 'fp64' or 'fp32'");
    }
    std::string getPrecision() const { return precision == IK_PREC_FP64 ? "fp64" : "fp32"; }
    void compute(py::handle gridpoints)
    {
        std::vector<double> grid = to_xyz(gridpoints, (size_t)-1, "gridpoints");
        int64_t G = (int64_t)grid.size() / 3;
        const int kind = pot->model();
        if (ik_potential_nparams(kind) < 0)
            throw std::invalid_argument("[ERROR]: the base PairPotential has no force model");
        if ((int)pot->params.size() < ik_potential_nparams(kind))
            throw std::invalid_argument("[ERROR]: too few pair-potential parameters");
        const SimBox& b = *sys->simbox;
        double L[3] = {b.boxsize[0], b.boxsize[1], b.boxsize[2]};
        double o[3] = {b.origin[0], b.origin[1], b.origin[2]};
        int fields = 0;
        for (auto& kv : obs) {
            if (kv.second->dim != b.dim) throw std::invalid_argument("[ERROR]: observable dimension != box dimension");
            if ((int64_t)kv.second->val.size() != G * b.dim * b.dim)
                throw std::invalid_argument("[ERROR]: observable gridsize != number of grid points");
            fields |= kv.second->field;
        }
        if (!fields) return;
        {
            py::gil_scoped_release nogil;
            check(ik_set_box(ctx, b.dim, L, o));
            check(ik_set_potential(ctx, kind, pot->scaled_rcut, pot->params.data(), (int)pot->params.size()));
            cg->apply(ctx);
            check(ik_set_max_rcut(ctx, max_rcut));
            if (grid != last_grid) {
                check(ik_set_grid(ctx, G, grid.data()));
                last_grid = grid;
            }
            if (uploaded != sys->version || uploaded_sys != sys.get()) {
                check(ik_set_frame(ctx, sys->N, sys->pos.data(), sys->vel.data(), sys->mass.data(),
                                   sys->diameter.data()));
                uploaded = sys->version;
                uploaded_sys = sys.get();
            }
            if (fields & IK_FIELD_ELASTIC) // ParticleSystem::setDisplacement (ParticleSystem.cc:60-67)
                check(ik_upload_displacement(ctx, 0, sys->N, sys->disp.data()));
            check(ik_compute(ctx, precision, fields));
            for (auto& kv : obs)
                check(ik_get_field(ctx, 0, kv.second->field, kv.second->val.data(), (int64_t)kv.second->val.size()));
        }
    }
    std::vector<int64_t> counters()
    {
        std::vector<int64_t> c(3, 0);
        check(ik_get_counters(ctx, 0, c.data()));
        return c;
    }
};

// ---------------------------------------------------------------- _thermo
// Global observables (thermo/ThermoProperty.h, thermo/module-thermo.cpp:7-20): the value
// tensor of one part of ik_compute_thermo's output, saved as std::to_string(val[index]).
enum { TH_ENERGY = 0, TH_VIRIAL = 1, TH_ELASTIC = 2, TH_KINETIC = 3, TH_BORN = 4 };
struct ThermoProperty {
    std::string name, type;
    bool islocal = false;
    int dim = 2, part = TH_ENERGY;
    std::vector<double> val;
    ThermoProperty(std::string n, std::string t, bool local, int d, int pt)
        : name(std::move(n)), type(std::move(t)), islocal(local), dim(d), part(pt)
    {
        const size_t D2 = (size_t)d * d;
        val.assign(pt == TH_ENERGY ? 1 : (pt == TH_BORN ? D2 * D2 : D2), 0.0);
    }
    virtual ~ThermoProperty() = default;
    void save(MPILogFile& f, int index)
    {
        if (index < 0 || (size_t)index >= val.size()) throw std::out_of_range("[ERROR]: component index out of range");
        f.write_shared(std::to_string(val[(size_t)index]));
    }
    void clear() { std::fill(val.begin(), val.end(), 0.0); }
    // the part's slice of ik_compute_thermo's output
    void take(const std::vector<double>& out)
    {
        const size_t D2 = (size_t)dim * dim;
        const size_t off = part == TH_ENERGY ? 0 : (part == TH_BORN ? 1 + 3 * D2 : 1 + (size_t)(part - 1) * D2);
        std::copy(out.begin() + (long)off, out.begin() + (long)(off + val.size()), val.begin());
    }
};

template <int D, int PART>
struct GlobalProperty : ThermoProperty {
    GlobalProperty(std::string n, std::string t, bool local) : ThermoProperty(std::move(n), std::move(t), local, D, PART) {}
};

// ThermoCalculator (thermo/ThermoCalculator.h:7-90): max_rcut frozen at construction as
// Calculator does (Calculator.h:41-45); compute() fills every added observable.
struct ThermoCalculator {
    std::shared_ptr<ParticleSystem> sys;
    std::shared_ptr<PairPotential> pot;
    std::map<std::string, std::shared_ptr<ThermoProperty>> obs;
    ik_ctx* ctx = nullptr;
    double max_rcut = 0.0;
    uint64_t uploaded = (uint64_t)-1;
    const ParticleSystem* uploaded_sys = nullptr;

    ThermoCalculator(std::shared_ptr<ParticleSystem> s, std::shared_ptr<PairPotential> p)
        : sys(std::move(s)), pot(std::move(p))
    {
        if (!sys || !pot) throw std::invalid_argument("[ERROR]: ThermoCalculator needs sysdata and a potential");
        double dmax = 0.0;
        for (double d : sys->diameter) dmax = std::max(dmax, d);
        max_rcut = std::max(pot->scaled_rcut * dmax, dmax);
        check(ik_create(&ctx, 0));
    }
    ~ThermoCalculator() { if (ctx) ik_destroy(ctx); }
    void setSystemData(std::shared_ptr<ParticleSystem> s) { sys = std::move(s); }
    void addObservable(std::shared_ptr<ThermoProperty> o) { obs[o->name] = std::move(o); }
    void compute()
    {
        const int kind = pot->model();
        if (ik_potential_nparams(kind) < 0) throw std::invalid_argument("[ERROR]: the base PairPotential has no force model");
        if ((int)pot->params.size() < ik_potential_nparams(kind))
            throw std::invalid_argument("[ERROR]: too few pair-potential parameters");
        const SimBox& b = *sys->simbox;
        std::vector<double> out((size_t)(1 + 3 * b.dim * b.dim + b.dim * b.dim * b.dim * b.dim));
        {
            py::gil_scoped_release nogil;
            double L[3] = {b.boxsize[0], b.boxsize[1], b.boxsize[2]};
            double o[3] = {b.origin[0], b.origin[1], b.origin[2]};
            check(ik_set_box(ctx, b.dim, L, o));
            check(ik_set_potential(ctx, kind, pot->scaled_rcut, pot->params.data(), (int)pot->params.size()));
            check(ik_set_max_rcut(ctx, max_rcut));
            if (uploaded != sys->version || uploaded_sys != sys.get()) {
                check(ik_set_frame(ctx, sys->N, sys->pos.data(), sys->vel.data(), sys->mass.data(),
                                   sys->diameter.data()));
                uploaded = sys->version;
                uploaded_sys = sys.get();
            }
            bool ela = false;
            for (auto& kv : obs) ela = ela || kv.second->part == TH_ELASTIC;
            if (ela) check(ik_upload_displacement(ctx, 0, sys->N, sys->disp.data()));
            check(ik_compute_thermo(ctx, 0, out.data(), (int64_t)out.size()));
        }
        for (auto& kv : obs) {
            if (kv.second->dim != b.dim) throw std::invalid_argument("[ERROR]: observable dimension != box dimension");
            kv.second->take(out);
        }
    }
};

// ---------------------------------------------------------------- module
// export_ThermoProperty (thermo/ThermoProperty.h:217-225)
template <int D, int PART>
static void export_thermo_property(py::module& tm, const char* name)
{
    using T = GlobalProperty<D, PART>;
    py::class_<T, ThermoProperty, std::shared_ptr<T>>(tm, name)
        .def(py::init<std::string, std::string, bool>())
        .def("save", &T::save)
        .def("clear", &T::clear);
}

// export_ShortRangePairPotential (potential/PairPotential.h:139-152)
template <int KIND>
static void export_short_range(py::module& pm, const char* name)
{
    using T = ShortRangePairPotential<KIND>;
    py::class_<T, PairPotential, std::shared_ptr<T>>(pm, name)
        .def(py::init<std::vector<double>>())
        .def(py::init<double, std::vector<double>>())
        .def("getRcut", &T::getRcut)
        .def("getPairForceDivR", &T::getPairForceDivR)
        .def("getPairEnergy", &T::getPairEnergy)
        .def("getParams", &T::getParams)
        .def("setParams", &T::setParams)
        .def_readwrite("scaled_rcut", &T::scaled_rcut);
}

PYBIND11_MODULE(_core, m)
{
    m.doc() = "GB300 Irving-Kirkwood engine: pybind11 mirror of pyglasstools' native modules";
    m.def("abi_version", &ik_version);

    py::module pg = m.def_submodule("_pyglasstools");
    py::class_<SimBox, std::shared_ptr<SimBox>>(pg, "SimBox")
        .def(py::init([](double L, py::handle o, int d) { return std::make_shared<SimBox>(Vec3{L, L, L}, to3(o), d); }))
        .def(py::init([](py::handle L, py::handle o, int d) { return std::make_shared<SimBox>(to3(L), to3(o), d); }))
        .def("minImage", &SimBox::minImage)
        .def_readwrite("dim", &SimBox::dim)
        .def_readwrite("origin", &SimBox::origin)
        .def_readwrite("boxsize", &SimBox::boxsize)
        .def_readwrite("upperbound", &SimBox::upperbound)
        .def_readwrite("lowerbound", &SimBox::lowerbound)
        .def_readwrite("periodic", &SimBox::periodic)
        .def_readwrite("vol", &SimBox::vol);
    py::class_<ParticleSystem, std::shared_ptr<ParticleSystem>>(pg, "ParticleSystem")
        .def(py::init<std::shared_ptr<SimBox>, unsigned int, py::handle, py::handle, py::handle, py::handle>())
        .def("getMass", [](ParticleSystem& s) { return s.mass; })
        .def("setMass", [](ParticleSystem& s, py::handle m) {
            auto v = to_vec(m, "mass");
            if (v.size() != s.N) throw std::invalid_argument("[ERROR]: Size of mass array mismatch with # of particles!");
            s.mass = v; ++s.version; })
        .def("getDiameter", [](ParticleSystem& s) { return s.diameter; })
        .def("setDiameter", [](ParticleSystem& s, py::handle d) {
            auto v = to_vec(d, "diameter");
            if (v.size() != s.N) throw std::invalid_argument("[ERROR]: Size of diameter array mismatch with # of particles!");
            s.diameter = v; ++s.version; })
        .def("getDisplacement", [](ParticleSystem& s) { return ParticleSystem::as_nx3(s.disp); })
        .def("setDisplacement", [](ParticleSystem& s, py::handle d) { s.disp = to_xyz(d, s.N, "displacement"); })
        .def("setAtomPosition", [](ParticleSystem& s, py::handle p) { s.pos = to_xyz(p, s.N, "position"); ++s.version; })
        .def("setAtomVelocity", [](ParticleSystem& s, py::handle v) { s.vel = to_xyz(v, s.N, "velocity"); ++s.version; })
        .def("getAtomPosition", [](ParticleSystem& s) { return ParticleSystem::as_nx3(s.pos); })
        .def("getAtomVelocity", [](ParticleSystem& s) { return ParticleSystem::as_nx3(s.vel); })
        .def("moveParticles", [](ParticleSystem& s, py::handle p) {
            auto d = to_xyz(p, s.N, "position");
            for (size_t k = 0; k < d.size(); ++k) s.pos[k] += d[k];
            ++s.version; })
        .def("moveParticles", [](ParticleSystem& s) {
            for (size_t k = 0; k < s.pos.size(); ++k) s.pos[k] += s.disp[k];
            ++s.version; })
        .def("getNeighbors", &ParticleSystem::getNeighbors)
        .def("getNeighborsDistance", &ParticleSystem::getNeighborsDistance)
        .def("neighborList", &ParticleSystem::neighborList)
        .def("update", [](ParticleSystem& s, unsigned int n, py::handle d, py::handle m, py::handle p, py::handle v) {
            s.set(n, d, m, p, v); })
        .def_readonly("N", &ParticleSystem::N)
        .def_readonly("simbox", &ParticleSystem::simbox);
    py::class_<Communicator, std::shared_ptr<Communicator>>(pg, "Communicator")
        .def(py::init<>())
        .def("getRank", &Communicator::getRank)
        .def("getSizeGlobal", &Communicator::getSizeGlobal)
        .def("barrier", &Communicator::barrier)
        .def("abort", &Communicator::abort)
        .def("bcast", &Communicator::bcast)
        .def("scatter_v", &Communicator::scatter_v)
        .def("gather_v", &Communicator::gather_v)
        .def("all_gather_v", &Communicator::all_gather_v)
        .def("send", &Communicator::send)
        .def("recv", &Communicator::recv);
    py::class_<MPILogFile, std::shared_ptr<MPILogFile>>(pg, "MPILogFile")
        .def(py::init<std::shared_ptr<Communicator>, const std::string&>())
        .def("write_shared", &MPILogFile::write_shared)
        .def("flush", &MPILogFile::flush)
        .def("close", &MPILogFile::close);
    py::class_<Manager, std::shared_ptr<Manager>>(pg, "Manager")
        .def(py::init<>())
        .def_readwrite("notice_level", &Manager::notice_level);

    py::module pm = m.def_submodule("_potential");
    py::class_<PairPotential, std::shared_ptr<PairPotential>>(pm, "PairPotential")
        .def(py::init<std::vector<double>>())
        .def(py::init<double, std::vector<double>>())
        .def("getRcut", &PairPotential::getRcut)
        .def("getPairForceDivR", &PairPotential::getPairForceDivR)
        .def("getPairEnergy", &PairPotential::getPairEnergy)
        .def("getParams", &PairPotential::getParams)
        .def("setParams", &PairPotential::setParams)
        .def_readwrite("scaled_rcut", &PairPotential::scaled_rcut);
    export_short_range<IK_POT_LJ>(pm, "PairPotentialLJ");
    export_short_range<IK_POT_FSLJ>(pm, "PairPotentialForceShiftedLJ");
    export_short_range<IK_POT_POLY12>(pm, "PairPotentialPoly12");
    export_short_range<IK_POT_POLY18>(pm, "PairPotentialPoly18");
    export_short_range<IK_POT_POLY10>(pm, "PairPotentialPoly10");
    export_short_range<IK_POT_POLY106>(pm, "PairPotentialPoly106");
    export_short_range<IK_POT_POLYYUKAWA>(pm, "PairPotentialPolyYukawa");
    export_short_range<IK_POT_POLYLJ>(pm, "PairPotentialPolyLJ");

    py::module tm = m.def_submodule("_thermo");
    py::class_<ThermoCalculator, std::shared_ptr<ThermoCalculator>>(tm, "ThermoCalculator")
        .def(py::init<std::shared_ptr<ParticleSystem>, std::shared_ptr<PairPotential>>())
        .def("compute", &ThermoCalculator::compute)
        .def("setSystemData", &ThermoCalculator::setSystemData)
        .def("addObservable", &ThermoCalculator::addObservable)
        .def_readonly("max_rcut", &ThermoCalculator::max_rcut);
    py::class_<ThermoProperty, std::shared_ptr<ThermoProperty>>(tm, "ThermoProperty")
        .def_readonly("name", &ThermoProperty::name)
        .def_readonly("type", &ThermoProperty::type)
        .def_readonly("islocal", &ThermoProperty::islocal)
        .def_readonly("dim", &ThermoProperty::dim)
        .def_property_readonly("val", [](const ThermoProperty& t) { return t.val; });
    export_thermo_property<2, TH_ENERGY>(tm, "GlobalPotentialEnergy2D");
    export_thermo_property<3, TH_ENERGY>(tm, "GlobalPotentialEnergy3D");
    export_thermo_property<2, TH_VIRIAL>(tm, "GlobalVirialStress2D");
    export_thermo_property<3, TH_VIRIAL>(tm, "GlobalVirialStress3D");
    export_thermo_property<2, TH_ELASTIC>(tm, "GlobalElasticVirialStress2D");
    export_thermo_property<3, TH_ELASTIC>(tm, "GlobalElasticVirialStress3D");
    export_thermo_property<2, TH_BORN>(tm, "GlobalBornTensor2D");
    export_thermo_property<3, TH_BORN>(tm, "GlobalBornTensor3D");
    export_thermo_property<2, TH_KINETIC>(tm, "GlobalKineticStress2D");
    export_thermo_property<3, TH_KINETIC>(tm, "GlobalKineticStress3D");

    py::module cm = m.def_submodule("_cgfunc");
    py::class_<CoarseGrainFunction, std::shared_ptr<CoarseGrainFunction>>(cm, "CoarseGrainFunction")
        .def(py::init<double>())
        .def("getRcut", &CoarseGrainFunction::getRcut)
        .def("setRcut", &CoarseGrainFunction::setRcut)
        .def("getDeltaFunc", &CoarseGrainFunction::getDeltaFunc)
        .def("getObjFunc", &CoarseGrainFunction::getObjFunc)
        .def("getBondFunc", &CoarseGrainFunction::getBondFunc)
        .def_property_readonly("mode", [](const CoarseGrainFunction& f) {
            return std::string(f.mode == IK_QUAD_ADAPTIVE ? "adaptive" : f.mode == IK_QUAD_EXACT ? "exact"
                               : f.mode == IK_QUAD_MLP ? "mlp" : "fixedpoint");
        });
#define FIXED(T, NAME) py::class_<T, CoarseGrainFunction, std::shared_ptr<T>>(cm, NAME).def(py::init<int, double>())
#define ADAPT(T, NAME) \
    py::class_<T, CoarseGrainFunction, std::shared_ptr<T>>(cm, NAME).def(py::init<int, double, double, double>())
    FIXED(CGFixed<IK_CG_OCTIC>, "CGFuncOcticFixedPoint");
    ADAPT(CGAdaptive<IK_CG_OCTIC>, "CGFuncOcticAdaptive");
    FIXED(CGFixed<IK_CG_RECT>, "CGFuncRectFixedPoint");
    ADAPT(CGAdaptive<IK_CG_RECT>, "CGFuncRectAdaptive");
    FIXED(CGFixed<IK_CG_MOLLIFIER>, "CGFuncMollifierFixedPoint");
    ADAPT(CGAdaptive<IK_CG_MOLLIFIER>, "CGFuncMollifierAdaptive");
#undef FIXED
#undef ADAPT
    py::class_<CGGaussianFixed, CoarseGrainFunction, std::shared_ptr<CGGaussianFixed>>(cm, "CGFuncGaussianFixedPoint")
        .def(py::init<int, double, double>(), py::arg("order"), py::arg("width"), py::arg("cut") = 3.0);
    py::class_<CGGaussianAdaptive, CoarseGrainFunction, std::shared_ptr<CGGaussianAdaptive>>(cm,
                                                                                           "CGFuncGaussianAdaptive")
        .def(py::init<int, double, double, double, double>(), py::arg("neval"), py::arg("relerr"),
             py::arg("abserr"), py::arg("width"), py::arg("cut") = 3.0);

    py::module im = m.def_submodule("_irvingkirkwood");
    py::class_<IrvingKirkwood, std::shared_ptr<IrvingKirkwood>>(im, "IrvingKirkwood")
        .def(py::init<std::shared_ptr<ParticleSystem>, std::shared_ptr<PairPotential>,
                      std::shared_ptr<CoarseGrainFunction>, std::shared_ptr<Communicator>>())
        .def("compute", &IrvingKirkwood::compute)
        .def("setSystemData", &IrvingKirkwood::setSystemData)
        .def("addObservable", &IrvingKirkwood::addObservable)
        .def("printDisplacement", &IrvingKirkwood::printDisplacement)
        .def("setPrecision", &IrvingKirkwood::setPrecision)
        .def("getPrecision", &IrvingKirkwood::getPrecision)
        .def("counters", &IrvingKirkwood::counters)
        .def_readonly("max_rcut", &IrvingKirkwood::max_rcut);
    py::class_<CoarseGrainedField, std::shared_ptr<CoarseGrainedField>>(im, "CoarseGrainedField")
        .def("addGridpoints", &CoarseGrainedField::addGridpoints)
        .def("gettostring", &CoarseGrainedField::gettostring)
        .def("save", &CoarseGrainedField::save)
        .def("clear", &CoarseGrainedField::clear)
        .def("values", &CoarseGrainedField::values)
        .def_readonly("name", &CoarseGrainedField::name)
        .def_readonly("type", &CoarseGrainedField::type)
        .def_readonly("islocal", &CoarseGrainedField::islocal)
        .def_readonly("dim", &CoarseGrainedField::dim);
    // Lines of one frame of fieldlogger.save_perrank / save_perrank_polar (io.py:112-144):
    // per grid point "1 " + the leading columns (repr) + each requested component of
    // each field (gettostring: default ostream, 6 significant digits) + "\n".
    im.def("format_field_lines",
           [](py::array_t<double, py::array::c_style | py::array::forcecast> cols,
              const std::vector<std::pair<std::shared_ptr<CoarseGrainedField>, int>>& comps,
              const std::vector<int>& int_cols) {
               auto c = cols.unchecked<2>();
               const py::ssize_t G = c.shape(0), K = c.shape(1);
               for (auto& fc : comps) {
                   const size_t DD = (size_t)fc.first->dim * fc.first->dim;
                   if (fc.second < 0 || (size_t)fc.second >= DD || fc.first->val.size() < (size_t)G * DD)
                       throw std::out_of_range("[ERROR]: grid/component index out of range");
               }
               std::string out;
               out.reserve((size_t)G * (16 * (size_t)K + 14 * comps.size() + 4));
               char vb[64];
               {
                   py::gil_scoped_release nogil;
                   for (py::ssize_t g = 0; g < G; ++g) {
                       out += "1 ";
                       for (py::ssize_t k = 0; k < K; ++k) {
                           if (std::find(int_cols.begin(), int_cols.end(), (int)k) != int_cols.end()) {
                               std::snprintf(vb, sizeof vb, "%lld", (long long)c(g, k));
                               out += vb;
                           } else {
                               py_float_repr(c(g, k), out);
                           }
                           out += ' ';
                       }
                       for (auto& fc : comps) {
                           const size_t DD = (size_t)fc.first->dim * fc.first->dim;
                           std::snprintf(vb, sizeof vb, "%g ", fc.first->val[(size_t)g * DD + (size_t)fc.second]);
                           out += vb;
                       }
                       out += '\n';
                   }
               }
               return out;
           },
           py::arg("cols"), py::arg("comps"), py::arg("int_cols") = std::vector<int>{});
    im.def("float_repr", [](double v) { std::string o; py_float_repr(v, o); return o; });
#define FIELD(D, F, NAME)                                                                    \
    py::class_<FieldT<D, F>, CoarseGrainedField, std::shared_ptr<FieldT<D, F>>>(im, NAME) \
        .def(py::init<std::string, std::string, bool, int>())
    FIELD(2, IK_FIELD_VIRIAL, "VirialStressField2D");
    FIELD(3, IK_FIELD_VIRIAL, "VirialStressField3D");
    FIELD(2, IK_FIELD_KINETIC, "KineticStressField2D");
    FIELD(3, IK_FIELD_KINETIC, "KineticStressField3D");
    FIELD(2, IK_FIELD_ELASTIC, "ElasticVirialStressField2D");
    FIELD(3, IK_FIELD_ELASTIC, "ElasticVirialStressField3D");
#undef FIELD
}
