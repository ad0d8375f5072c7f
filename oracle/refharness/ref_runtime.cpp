// Minimal stand-ins for the parts of liblightmetrica that the reference's
// accel / renderer sources call through LM_EXPORTED_F, so that those sources
// can be compiled unmodified as a CPU oracle.  Only this container builds it:
// the reference's component.cpp and logger.cpp need boost/TBB, which are absent.
//
// Behaviour mirrored (written here, not copied):
//   ComponentFactory_*  -> src/liblightmetrica/component.cpp:56-104
//                         (map key -> create/release, Create stamps createKey)
//   Logger_*            -> src/liblightmetrica/logger.cpp (messages to stderr)
#include <pch.h>
#include <lightmetrica/component.h>
#include <lightmetrica/logger.h>
#include <lightmetrica/exception.h>
#include <lightmetrica/debug.h>

#include <map>

LM_NAMESPACE_BEGIN

namespace {
struct FactoryEntry { CreateFuncPointerType create; ReleaseFuncPointerType release; };
std::map<std::string, FactoryEntry>& Registry()
{
    static std::map<std::string, FactoryEntry> m;
    return m;
}
int g_verbose = 0;
}

extern "C" {

LM_PUBLIC_API auto ComponentFactory_Register(const char* key, CreateFuncPointerType createFunc, ReleaseFuncPointerType releaseFunc) -> void
{
    auto& r = Registry();
    if (r.count(key)) std::cerr << "duplicate registration: " << key << std::endl;
    r[key] = FactoryEntry{ createFunc, releaseFunc };
}

LM_PUBLIC_API auto ComponentFactory_Unregister(const char* key) -> void { Registry().erase(key); }

LM_PUBLIC_API auto ComponentFactory_Create(const char* key) -> Component*
{
    auto& r = Registry();
    auto it = r.find(key);
    if (it == r.end()) return nullptr;
    Component* p = it->second.create();
    p->createFunc = it->second.create;
    p->releaseFunc = it->second.release;
    p->createKey = it->first.c_str();
    return p;
}

LM_PUBLIC_API auto ComponentFactory_ReleaseFunc(const char* key) -> ReleaseFuncPointerType
{
    auto& r = Registry();
    auto it = r.find(key);
    return it == r.end() ? nullptr : it->second.release;
}

LM_PUBLIC_API auto ComponentFactory_LoadPlugin(const char*) -> bool { return false; }
LM_PUBLIC_API auto ComponentFactory_LoadPlugins(const char*) -> void {}
LM_PUBLIC_API auto ComponentFactory_UnloadPlugins() -> void {}

LM_PUBLIC_API auto Logger_Run() -> void {}
LM_PUBLIC_API auto Logger_Stop() -> void {}
LM_PUBLIC_API auto Logger_SetVerboseLevel(int level) -> void { g_verbose = level; }
LM_PUBLIC_API auto Logger_Log(int type, const char* message, const char* filename, int line, bool, bool) -> void
{
    // type: 0 error, 1 warn, 2 info, 3 debug (logger.h LogType order)
    if (type <= 1 || g_verbose > 0)
        std::fprintf(stderr, "[ref %d] %s (%s:%d)\n", type, message, filename ? filename : "?", line);
}
LM_PUBLIC_API auto Logger_UpdateIndentation(bool) -> void {}
LM_PUBLIC_API auto Logger_Flush() -> void {}

LM_PUBLIC_API auto DebugUtils_StackTrace() -> bool { return false; }
LM_PUBLIC_API auto SEHUtils_EnableStructuralException() -> void {}
LM_PUBLIC_API auto SEHUtils_DisableStructuralException() -> void {}

}

LM_NAMESPACE_END
