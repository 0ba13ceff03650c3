// libaqua_cuda_tool.so -- installable tools that run the canonical WCSPH
// step, or only its link-list, on the GPU through the aqua_gb300 C ABI.  They
// have the shape of the reference's installable-tool example
// (tests/ExternalTool/tool.{hpp,cpp}: a Tool subclass plus a C-linkage
// create_object(name, once) factory), so a step loop can name the library
// in a <Tool type="installable" path="libaqua_cuda_tool.so"> element:
//
//   - a tool named "link-list..." replaces the link-list tool
//     (LinkList.cpp:326-494): r_in in; icell, id_sorted, id_unsorted, ihoc,
//     n_cells, r_min, r_max out;
//   - any other name replaces the tools from "predictor" to "iter += 1"
//     (basic.xml:132-171 with the midpoint, domain, cfd, deltaSPH, BIe and
//     variableTimeStep presets): setup() reads the case's Variables and
//     Definitions and creates the device context; every execution uploads
//     the particle Variables, runs one step, checks it and downloads the
//     Variables and the scalars t, dt, iter.
#include <cstring>
#include <string>
#include <vector>

#include "aqua_gb300.h"
#include "aqua_host.hpp"

namespace {

std::string
status_text(const char* what, aqua_status s)
{
    return std::string(what) + " returned status " + std::to_string((int)s);
}

}  // namespace

namespace aqua_host {

class AquaCudaStep : public Tool
{
  public:
    AquaCudaStep(const std::string tool_name, bool once)
      : Tool(tool_name, once)
    {
    }
    ~AquaCudaStep() override
    {
        if (_ctx)
            aqua_destroy(_ctx);
    }

    void setup() override
    {
        // the particle Variables the step reads and writes, and the scalars
        std::vector<std::string> io = { "N", "id", "iset", "imove", "r",
                                        "normal", "tangent", "u", "dudt", "rho",
                                        "drhodt", "m", "p", "t", "dt", "iter" };
        std::vector<std::string> in = io;
        for (const char* n : kCaseInputs)
            in.push_back(n);
        setDependencies(in, io);
        Tool::setup();

        aqua_params p;
        std::memset(&p, 0, sizeof(p));
        p.dims = scalar<int32_t>("dims");
        p.n_sets = scalar<uint32_t>("n_sets");
        p.h = scalar<float>("h");
        p.support = scalar<float>("support");
        p.H = scalar<float>("H");
        p.CONW = scalar<float>("CONW");
        p.CONF = scalar<float>("CONF");
        p.SUPPORT = scalar<float>("SUPPORT");
        p.DIMS = scalar<float>("DIMS");
        p.cs = scalar<float>("cs");
        p.p0 = scalar<float>("p0");
        vector4("g", p.g);
        p.courant = scalar<float>("courant");
        p.dt_Ma = scalar<float>("dt_Ma");
        p.dt_min = scalar<float>("dt_min");
        p.dt_fixed = scalar<float>("dt_fixed");
        vector4("domain_min", p.domain_min);
        vector4("domain_max", p.domain_max);
        p.dr_factor = scalar<float>("__DR_FACTOR__");
        p.min_bound_dist = scalar<float>("__MIN_BOUND_DIST__");
        p.relax_midpoint = scalar<float>("relax_midpoint");
        p.iter_midpoint_max = scalar<uint32_t>("iter_midpoint_max");
        p.refd = array<float>("refd", p.n_sets);
        p.visc_dyn = array<float>("visc_dyn", p.n_sets);
        p.delta = array<float>("delta", p.n_sets);
        p.boundary = variables().has("boundary") ? scalar<int32_t>("boundary")
                                                 : AQUA_BOUNDARY_BIE;
        p.scheme = variables().has("scheme") ? scalar<int32_t>("scheme")
                                             : AQUA_SCHEME_MIDPOINT;
        _n = scalar<uint32_t>("N");
        _vs = (p.dims == 3) ? 4 : 2;
        if (_ctx) {
            aqua_destroy(_ctx);
            _ctx = nullptr;
        }
        const aqua_status s = aqua_create(&p, _n, 0, &_ctx);
        if (s != AQUA_OK)
            throw std::runtime_error(status_text("aqua_create", s));
        if (variables().has("aqua_precision")) {
            const aqua_status q = aqua_set_precision(
                _ctx, scalar<int32_t>("aqua_precision"));
            if (q != AQUA_OK)
                throw std::runtime_error(status_text("aqua_set_precision", q));
        }
    }

  protected:
    void _execute() override
    {
        aqua_vars v;
        std::memset(&v, 0, sizeof(v));
        v.id = array<uint32_t>("id", _n);
        v.iset = array<uint32_t>("iset", _n);
        v.imove = array<int32_t>("imove", _n);
        v.r = array<float>("r", (size_t)_n * _vs);
        v.normal = array<float>("normal", (size_t)_n * _vs);
        v.tangent = array<float>("tangent", (size_t)_n * _vs);
        if (variables().has("binormal"))
            v.binormal = array<float>("binormal", (size_t)_n * _vs);
        v.u = array<float>("u", (size_t)_n * _vs);
        v.dudt = array<float>("dudt", (size_t)_n * _vs);
        v.rho = array<float>("rho", _n);
        v.drhodt = array<float>("drhodt", _n);
        v.m = array<float>("m", _n);
        v.p = array<float>("p", _n);
        check("aqua_set_state",
              aqua_set_state(_ctx, _n, &v, 1, scalar<float>("t"),
                             scalar<float>("dt"), scalar<uint32_t>("iter"),
                             nullptr));
        check("aqua_step", aqua_step(_ctx, 1, 1, nullptr));
        check("aqua_check", aqua_check(_ctx, nullptr));
        if (variables().has("shepard"))
            v.shepard = array<float>("shepard", _n);
        check("aqua_get_state", aqua_get_state(_ctx, &v, 1, nullptr));
        aqua_scalars sc;
        check("aqua_get_scalars", aqua_get_scalars(_ctx, &sc, nullptr));
        set_scalar<float>("t", sc.t);
        set_scalar<float>("dt", sc.dt);
        set_scalar<uint32_t>("iter", sc.iter);
    }

  private:
    // scalars, vectors and per-set arrays of the case
    static constexpr const char* kCaseInputs[] = {
        "dims", "n_sets", "h", "support", "H", "CONW", "CONF", "SUPPORT",
        "DIMS", "cs", "p0", "g", "courant", "dt_Ma", "dt_min", "dt_fixed",
        "domain_min", "domain_max", "__DR_FACTOR__", "__MIN_BOUND_DIST__",
        "relax_midpoint", "iter_midpoint_max", "refd", "visc_dyn", "delta"
    };

    Variable* sized(const std::string& name, size_t bytes)
    {
        Variable* v = variables().get(name);
        if (!v->data || v->bytes < bytes)
            throw std::runtime_error("Variable \"" + name + "\" holds " +
                                     std::to_string(v->bytes) + " bytes, " +
                                     std::to_string(bytes) + " needed");
        return v;
    }
    template<typename T>
    T scalar(const std::string& name)
    {
        T x;
        std::memcpy(&x, sized(name, sizeof(T))->data, sizeof(T));
        return x;
    }
    template<typename T>
    void set_scalar(const std::string& name, T x)
    {
        std::memcpy(sized(name, sizeof(T))->data, &x, sizeof(T));
    }
    template<typename T>
    T* array(const std::string& name, size_t count)
    {
        return static_cast<T*>(sized(name, count * sizeof(T))->data);
    }
    // a vec Variable: 2 floats in 2-D, 4 in 3-D (the rest stays 0)
    void vector4(const std::string& name, float out[4])
    {
        Variable* v = sized(name, 2 * sizeof(float));
        const size_t n = v->bytes >= 4 * sizeof(float) ? 4 : 2;
        std::memcpy(out, v->data, n * sizeof(float));
    }
    void check(const char* what, aqua_status s)
    {
        if (s != AQUA_OK)
            throw std::runtime_error(status_text(what, s));
    }

    aqua_ctx* _ctx = nullptr;
    uint32_t _n = 0;
    size_t _vs = 4;
};

// The link-list tool alone, on the registry's host Variables: r_in (vec*),
// N, h, support and dims in; icell, id_sorted, id_unsorted, ihoc (unsigned
// int*, ihoc sized for the cell capacity), n_cells (4 unsigned ints), r_min
// and r_max (vec) out.
class AquaCudaLinkList : public Tool
{
  public:
    AquaCudaLinkList(const std::string tool_name, bool once)
      : Tool(tool_name, once)
    {
    }
    ~AquaCudaLinkList() override { release(); }

    void setup() override
    {
        setDependencies({ "N", "dims", "h", "support", "r_in" },
                        { "icell", "id_sorted", "id_unsorted", "ihoc",
                          "n_cells", "r_min", "r_max" });
        Tool::setup();
        release();
        const int32_t dims = scalar<int32_t>(variables(), "dims");
        _n = scalar<uint32_t>(variables(), "N");
        _vs = dims == 3 ? 4 : 2;
        Variable* ih = variables().get("ihoc");
        _cap = (uint32_t)(ih->bytes / sizeof(uint32_t));
        // the link-list needs only h, support and the dimension; the other
        // parameters are placeholders the context validates
        static const float one = 1.f;
        aqua_params p;
        std::memset(&p, 0, sizeof(p));
        p.dims = dims;
        p.n_sets = 1;
        p.h = scalar<float>(variables(), "h");
        p.support = scalar<float>(variables(), "support");
        p.H = p.h;
        p.CONW = p.CONF = p.SUPPORT = p.DIMS = 1.f;
        p.refd = p.visc_dyn = p.delta = &one;
        p.iter_midpoint_max = 1;
        for (int k = 0; k < 4; k++) {
            p.domain_min[k] = -1.f;
            p.domain_max[k] = 1.f;
        }
        check("aqua_create", aqua_create(&p, _n, _cap, &_ctx));
        const size_t nb = (size_t)_n * sizeof(uint32_t);
        check("aqua_malloc", aqua_malloc(&_r, (size_t)_n * _vs * sizeof(float)));
        check("aqua_malloc", aqua_malloc(&_icell, nb));
        check("aqua_malloc", aqua_malloc(&_ids, nb));
        check("aqua_malloc", aqua_malloc(&_idu, nb));
        check("aqua_malloc", aqua_malloc(&_ihoc, (size_t)_cap * sizeof(uint32_t)));
    }

  protected:
    void _execute() override
    {
        Variables& v = variables();
        const size_t nb = (size_t)_n * sizeof(uint32_t);
        check("aqua_memcpy",
              aqua_memcpy(_r, array(v, "r_in", (size_t)_n * _vs * sizeof(float)),
                          (size_t)_n * _vs * sizeof(float), AQUA_COPY_H2D));
        uint32_t n_cells[4];
        float rmin[4], rmax[4];
        check("aqua_linklist",
              aqua_linklist(_ctx, static_cast<const float*>(_r), _n,
                            static_cast<uint32_t*>(_icell),
                            static_cast<uint32_t*>(_ids),
                            static_cast<uint32_t*>(_idu),
                            static_cast<uint32_t*>(_ihoc), _cap, n_cells, rmin,
                            rmax, nullptr));
        check("aqua_memcpy", aqua_memcpy(array(v, "icell", nb), _icell, nb,
                                         AQUA_COPY_D2H));
        check("aqua_memcpy", aqua_memcpy(array(v, "id_sorted", nb), _ids, nb,
                                         AQUA_COPY_D2H));
        check("aqua_memcpy", aqua_memcpy(array(v, "id_unsorted", nb), _idu, nb,
                                         AQUA_COPY_D2H));
        const size_t hb = (size_t)n_cells[3] * sizeof(uint32_t);
        check("aqua_memcpy", aqua_memcpy(array(v, "ihoc", hb), _ihoc, hb,
                                         AQUA_COPY_D2H));
        std::memcpy(array(v, "n_cells", sizeof(n_cells)), n_cells, sizeof(n_cells));
        std::memcpy(array(v, "r_min", _vs * sizeof(float)), rmin, _vs * sizeof(float));
        std::memcpy(array(v, "r_max", _vs * sizeof(float)), rmax, _vs * sizeof(float));
    }

  private:
    template<typename T>
    static T scalar(Variables& v, const std::string& name)
    {
        T x;
        std::memcpy(&x, array(v, name, sizeof(T)), sizeof(T));
        return x;
    }
    static void* array(Variables& v, const std::string& name, size_t bytes)
    {
        Variable* var = v.get(name);
        if (!var->data || var->bytes < bytes)
            throw std::runtime_error("Variable \"" + name + "\" holds " +
                                     std::to_string(var->bytes) + " bytes, " +
                                     std::to_string(bytes) + " needed");
        return var->data;
    }
    static void check(const char* what, aqua_status s)
    {
        if (s != AQUA_OK)
            throw std::runtime_error(status_text(what, s));
    }
    void release()
    {
        for (void** p : { &_r, &_icell, &_ids, &_idu, &_ihoc }) {
            aqua_free(*p);
            *p = nullptr;
        }
        if (_ctx) {
            aqua_destroy(_ctx);
            _ctx = nullptr;
        }
    }

    aqua_ctx* _ctx = nullptr;
    void *_r = nullptr, *_icell = nullptr, *_ids = nullptr, *_idu = nullptr,
         *_ihoc = nullptr;
    uint32_t _n = 0, _cap = 0;
    size_t _vs = 4;
};

}  // namespace aqua_host

// The factory the reference's CalcServer resolves with dlsym
// (CalcServer.cpp:388-398): C linkage, C++ std::string argument
extern "C" aqua_host::Tool*
create_object(const std::string name, bool once)
{
    if (name.compare(0, 9, "link-list") == 0)
        return new aqua_host::AquaCudaLinkList(name, once);
    return new aqua_host::AquaCudaStep(name, once);
}
