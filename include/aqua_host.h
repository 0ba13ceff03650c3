/*
 * aqua_host -- C entry points of the host runtime (libaqua_host.so) that
 * loads and runs installable step tools the way the reference's CalcServer
 * does (<Tool type="installable" path=...>, CalcServer.cpp:375-398).
 *
 * The runtime is one process-wide simulation: a registry of named host
 * Variables and an ordered tool list.  Every call returns 0 on success and
 * -1 on failure, with the reason in aqua_host_last_error() (the reference
 * throws std::runtime_error at the same points).
 */
#ifndef AQUA_HOST_H
#define AQUA_HOST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Registers (or re-points) the Variable `name` of reference type `type`
 * ("float", "vec", "unsigned int", "float*", "vec*", ...) at `data`, which
 * the caller keeps alive while the runtime uses it. */
int aqua_host_set_variable(const char* name, const char* type, void* data,
                           size_t bytes);

/* Loads the library at `path` (dlopen, RTLD_LAZY) and appends the tool its
 * create_object(name, once) builds; replaces the reference's parsing of
 * <Tool type="installable" name=... path=... once=...>. */
int aqua_host_add_installable(const char* name, const char* path, int once);

/* setup() of every tool in order (dependency checks, device resources). */
int aqua_host_setup(void);

/* `steps` passes over the tool list. */
int aqua_host_run(uint32_t steps);

/* Destroys the tools, closes their libraries and empties the registry. */
void aqua_host_clear(void);

/* Number of tools in the list. */
uint32_t aqua_host_tool_count(void);

/* Text of the last failure ("" if none). */
const char* aqua_host_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* AQUA_HOST_H */
