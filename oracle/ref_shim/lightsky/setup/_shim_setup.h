/*
 * Compatibility shim for LightSky's "setup" library (an absent submodule of
 * the reference tree), written for building the reference's draw-path
 * sources as a CPU oracle. Only what those sources use is provided. No
 * architecture macros (LS_X86_*, LS_ARM_*, LS_ARCH_*) are defined, so every
 * #if ladder in the reference takes its portable branch.
 */
#ifndef LS_SHIM_SETUP_H
#define LS_SHIM_SETUP_H

#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <thread>
#include <type_traits>
#include <utility>

#define LS_INLINE __attribute__((always_inline))
#define LS_IMPERATIVE
#define LS_API
#define LS_RESTRICT_PTR __restrict__
#define LS_LIKELY(x) __builtin_expect(!!(x), 1)
#define LS_UNLIKELY(x) __builtin_expect(!!(x), 0)
#define LS_UNREACHABLE() __builtin_unreachable()
#define LS_ARRAY_SIZE(a) (sizeof(a) / sizeof((a)[0]))
#define LS_ENUM_VAL(e) (static_cast<typename std::underlying_type<decltype(e)>::type>(e))
#define LS_PREFETCH(addr, rw, locality) __builtin_prefetch((addr), 0, 0)
#define LS_PREFETCH_ACCESS_R 0
#define LS_PREFETCH_ACCESS_RW 1
#define LS_PREFETCH_LEVEL_NONTEMPORAL 0
#define LS_PREFETCH_LEVEL_L1 3
#define LS_PREFETCH_LEVEL_L2 2
#define LS_PREFETCH_LEVEL_L3 1
#define LS_DECLARE_CLASS_TYPE(name, base, ...) typedef base<__VA_ARGS__> name
#define LS_DEFINE_CLASS_TYPE(base, ...) template class base<__VA_ARGS__>
#define LS_OS_LINUX 1
#define LS_OS_UNIX 1
#define LS_COMPILER_GNU 1

namespace ls
{
namespace setup
{

template <bool B, typename T = void> using EnableIf = std::enable_if<B, T>;
template <typename T> using IsIntegral = std::is_integral<T>;
template <typename T, typename U> using IsSame = std::is_same<T, U>;
template <typename T> using IsSigned = std::is_signed<T>;
template <typename B, typename D> using IsBaseOf = std::is_base_of<B, D>;
template <typename T> struct IsFloat : std::is_floating_point<T> {};
template <typename T> struct TrueType : std::true_type {};
template <typename T> struct FalseType : std::false_type {};
template <typename T> using RemoveRef = std::remove_reference<T>;
template <typename T> using RemoveConst = std::remove_const<T>;
template <typename T> using IsPointer = std::is_pointer<T>;

using std::forward;

inline void cpu_yield() noexcept { std::this_thread::yield(); }

} // namespace setup
} // namespace ls

#endif
