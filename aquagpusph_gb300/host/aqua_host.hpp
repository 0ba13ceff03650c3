// Host runtime for tools that drive the aqua_gb300 C ABI: the part of the
// reference's CalcServer that an installable tool sees.
//
//   - Variables: a registry of named host Variables (scalars, vectors and
//     per-particle arrays, with the reference's type names "float", "vec",
//     "unsigned int*", "vec*", ...), looked up by name as tools do through
//     CalcServer::singleton()->variables() (CalcServer.cpp).
//   - Tool: the interface of a step tool (aquagpusph/CalcServer/Tool.hpp:
//     162-372): constructed with (name, once), setup() checks and binds its
//     dependencies, execute() runs the protected _execute() (once-tools only
//     the first time).
//   - Runtime: the tool list of one simulation and the loader of installable
//     tools, which opens the library with dlopen(path, RTLD_LAZY) and builds
//     the tool with its C-linkage `create_object(const std::string, bool)`
//     factory, as CalcServer.cpp:375-398 does for
//     <Tool type="installable" path=...>.
//
// Variables live in host memory here (the reference keeps them in OpenCL
// buffers): a tool moves them to the device and back through the C ABI.
#pragma once

#include <cstddef>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace aqua_host {

// One named Variable in host memory, owned by whoever registered it
struct Variable
{
    std::string name;
    std::string type;
    void* data = nullptr;
    size_t bytes = 0;
};

class Variables
{
  public:
    // registers (or re-points) a Variable
    void set(const std::string& name, const std::string& type, void* data,
             size_t bytes);
    // the Variable; throws std::runtime_error naming it if it is missing
    Variable* get(const std::string& name);
    bool has(const std::string& name) const;
    void clear() { _vars.clear(); }

  private:
    std::map<std::string, Variable> _vars;
};

class Tool
{
  public:
    Tool(const std::string tool_name, bool once = false);
    virtual ~Tool();
    // checks that every dependency is registered (throws otherwise)
    virtual void setup();
    // runs _execute(); a once-tool runs only the first time
    void execute();
    const std::string& name() const { return _name; }
    bool once() const { return _once; }
    const std::vector<std::string>& inputs() const { return _inputs; }
    const std::vector<std::string>& outputs() const { return _outputs; }

  protected:
    virtual void _execute() = 0;
    // the Variables the tool reads and writes, by name
    void setDependencies(std::vector<std::string> inputs,
                         std::vector<std::string> outputs);
    // the simulation's registry
    Variables& variables();

  private:
    std::string _name;
    bool _once;
    bool _done = false;
    std::vector<std::string> _inputs, _outputs;
};

class Runtime
{
  public:
    static Runtime& singleton();
    Variables& variables() { return _vars; }
    // appends an installable tool built by the library's create_object()
    void add_installable(const std::string& name, const std::string& path,
                         bool once);
    // setup() of every tool, in order
    void setup();
    // `steps` passes over the tool list
    void run(unsigned steps);
    // destroys the tools, closes their libraries and empties the registry
    void clear();
    size_t n_tools() const { return _tools.size(); }

  private:
    Runtime() = default;
    ~Runtime();
    Variables _vars;
    std::vector<std::unique_ptr<Tool>> _tools;
    std::vector<void*> _handles;
};

}  // namespace aqua_host
