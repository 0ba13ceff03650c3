// Host runtime (libaqua_host.so): Variables registry, Tool base class and the
// installable-tool loader.  See aqua_host.hpp.
#include "aqua_host.hpp"

#include <dlfcn.h>

#include <sstream>
#include <string>

#include "aqua_host.h"

namespace aqua_host {

void
Variables::set(const std::string& name, const std::string& type, void* data,
               size_t bytes)
{
    Variable& v = _vars[name];
    v.name = name;
    v.type = type;
    v.data = data;
    v.bytes = bytes;
}

Variable*
Variables::get(const std::string& name)
{
    auto it = _vars.find(name);
    if (it == _vars.end())
        throw std::runtime_error("Variable \"" + name + "\" is not registered");
    return &it->second;
}

bool
Variables::has(const std::string& name) const
{
    return _vars.count(name) != 0;
}

Tool::Tool(const std::string tool_name, bool once)
  : _name(tool_name)
  , _once(once)
{
}

Tool::~Tool() = default;

void
Tool::setup()
{
    for (const auto* list : { &_inputs, &_outputs })
        for (const auto& n : *list)
            if (!variables().has(n))
                throw std::runtime_error("tool \"" + _name +
                                         "\" depends on the unregistered "
                                         "Variable \"" + n + "\"");
}

void
Tool::execute()
{
    if (_once && _done)
        return;
    _execute();
    _done = true;
}

void
Tool::setDependencies(std::vector<std::string> inputs,
                      std::vector<std::string> outputs)
{
    _inputs = std::move(inputs);
    _outputs = std::move(outputs);
}

Variables&
Tool::variables()
{
    return Runtime::singleton().variables();
}

Runtime&
Runtime::singleton()
{
    static Runtime rt;
    return rt;
}

Runtime::~Runtime()
{
    clear();
}

void
Runtime::add_installable(const std::string& name, const std::string& path,
                         bool once)
{
    void* handle = dlopen(path.c_str(), RTLD_LAZY);
    if (!handle) {
        const char* why = dlerror();
        throw std::runtime_error("installable tool \"" + name +
                                 "\" failed loading \"" + path + "\" (" +
                                 (why ? why : "?") + ")");
    }
    using Maker = Tool* (*)(const std::string, bool);
    auto maker = reinterpret_cast<Maker>(dlsym(handle, "create_object"));
    if (!maker) {
        dlclose(handle);
        throw std::runtime_error("installable tool \"" + name +
                                 "\" failed loading the create_object symbol "
                                 "from \"" + path + "\"");
    }
    Tool* t = maker(name, once);
    if (!t) {
        dlclose(handle);
        throw std::runtime_error("create_object of \"" + path +
                                 "\" returned no tool");
    }
    _tools.emplace_back(t);
    _handles.push_back(handle);
}

void
Runtime::setup()
{
    for (auto& t : _tools)
        t->setup();
}

void
Runtime::run(unsigned steps)
{
    for (unsigned s = 0; s < steps; s++)
        for (auto& t : _tools)
            t->execute();
}

void
Runtime::clear()
{
    // the tools' code lives in the libraries: destroy them first
    _tools.clear();
    for (void* h : _handles)
        dlclose(h);
    _handles.clear();
    _vars.clear();
}

}  // namespace aqua_host

// ------------------------------------------------------------------ C API

namespace {

thread_local std::string last_error;

template<typename F>
int
guarded(F&& f)
{
    try {
        f();
        last_error.clear();
        return 0;
    } catch (const std::exception& e) {
        last_error = e.what();
    } catch (...) {
        last_error = "unknown exception";
    }
    return -1;
}

}  // namespace

extern "C" int
aqua_host_set_variable(const char* name, const char* type, void* data,
                       size_t bytes)
{
    return guarded([&] {
        if (!name || !type)
            throw std::runtime_error("a Variable needs a name and a type");
        aqua_host::Runtime::singleton().variables().set(name, type, data, bytes);
    });
}

extern "C" int
aqua_host_add_installable(const char* name, const char* path, int once)
{
    return guarded([&] {
        if (!name || !path)
            throw std::runtime_error("an installable tool needs a name and a path");
        aqua_host::Runtime::singleton().add_installable(name, path, once != 0);
    });
}

extern "C" int
aqua_host_setup(void)
{
    return guarded([] { aqua_host::Runtime::singleton().setup(); });
}

extern "C" int
aqua_host_run(uint32_t steps)
{
    return guarded([&] { aqua_host::Runtime::singleton().run(steps); });
}

extern "C" void
aqua_host_clear(void)
{
    guarded([] { aqua_host::Runtime::singleton().clear(); });
}

extern "C" uint32_t
aqua_host_tool_count(void)
{
    return (uint32_t)aqua_host::Runtime::singleton().n_tools();
}

extern "C" const char*
aqua_host_last_error(void)
{
    return last_error.c_str();
}
