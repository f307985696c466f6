// Minimal stand-in for the entt registry calls made by ShadowVoxSystem.cpp:
// view<...>().each(fn), prepare<T>(), on_destroy<T>().connect<&F>(obj), get<T>(e).
// Entities are visited in creation order. Component storage lives in the
// harness (found by argument-dependent lookup of shim_each / shim_get).
// Reference-build recipe only (test infrastructure).
#pragma once
#include <cstdint>
#include <functional>

namespace entt {
enum class entity : std::uint32_t {};
struct registry;
template <class... Ts>
struct basic_view {
    registry* r;
    template <class F>
    void each(F f) {
        shim_each(*r, f, static_cast<basic_view*>(nullptr));
    }
};
template <class T>
struct sink {
    registry* r;
    template <auto Fn, class I>
    void connect(I* inst);
};
struct registry {
    std::function<void(registry&, entity)> on_destroy_cb;
    template <class... Ts>
    basic_view<Ts...> view() {
        return basic_view<Ts...>{this};
    }
    template <class T>
    void prepare() {}
    template <class T>
    sink<T> on_destroy() {
        return sink<T>{this};
    }
    template <class T>
    T& get(entity e) {
        return shim_get(*this, e, static_cast<T*>(nullptr));
    }
};
template <class T>
template <auto Fn, class I>
void sink<T>::connect(I* inst) {
    r->on_destroy_cb = [inst](registry& reg, entity e) { (inst->*Fn)(reg, e); };
}
}  // namespace entt
