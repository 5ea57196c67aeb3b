/*
 * Compatibility stub for LightSky's "script" library (an absent submodule of
 * the reference tree): the scene-graph headers name a script class template
 * keyed by a string hash only to befriend it. Nothing is scripted here.
 */
#ifndef LS_SHIM_SCRIPT_H
#define LS_SHIM_SCRIPT_H

#include <cstdint>

namespace ls
{
namespace script
{
typedef uint64_t hash_t;
} // namespace script
} // namespace ls

#define LS_SCRIPT_HASH_FUNC(str) ((ls::script::hash_t)sizeof(str))

#endif /* LS_SHIM_SCRIPT_H */
