// Oracle (test infrastructure only): stand-in for the reference's lm/core.h.
//
// The reference's core headers bring in nlohmann_json, cereal and its component registry,
// logger and floating-point-exception control. The reference sources compiled into oracle/_ref
// use only a few names from them; this header gives those names with the behaviour the compiled
// code relies on, and the reference's own include/lm/math.h for the math layer:
//   * Component -- the polymorphic base of every interface;
//   * Json and json::value / comp_ref / comp_ref_or_nullptr -- component properties: a flat map
//     from names to numbers, number arrays (vectors) or strings (locators of components added
//     with refshim::add_named), as the compiled constructors read them;
//   * Component::construct / underlying / foreach_underlying and comp::visit -- the hooks the
//     compiled components override;
//   * LM_COMP_REG_IMPL(Impl, key) -- registers a factory under its key (lm::refshim::create);
//   * LM_SERIALIZE_IMPL(ar) -- opens a serialization template that is never instantiated;
//   * LM_INFO -- logging, dropped;
//   * Error and LM_THROW_EXCEPTION_DEFAULT -- errors, thrown as std::runtime_error;
//   * exception::ScopedDisableFPEx -- floating-point exceptions are never enabled in this library,
//     so the guard has nothing to do.
#pragma once
#include <pch.h>
#include <lm/math.h>

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

class Json {
public:
    struct Entry {
        std::vector<double> nums;
        std::string str;
        bool is_str = false;
        // a value read as a 4x4 matrix (16 numbers, column-major)
        operator Mat4() const {
            Mat4 m;
            for (int c = 0; c < 4; c++) m[c] = Vec4(nums.at(4 * c), nums.at(4 * c + 1), nums.at(4 * c + 2), nums.at(4 * c + 3));
            return m;
        }
    };
    // one name-value pair of a brace-initialised object ({"eye", position_}, {"vfov", vfov_})
    struct Item {
        std::string name;
        Entry e;
        Item(const char* n, double v) : name(n), e{{v}, {}, false} {}
        Item(const char* n, const Vec3& v) : name(n), e{{v.x, v.y, v.z}, {}, false} {}
    };
    std::map<std::string, Entry> entries;
    Json() = default;
    Json(std::initializer_list<Item> items) {
        for (const auto& it : items) entries[it.name] = it.e;
    }
    void set(const std::string& name, std::vector<double> v) { entries[name] = Entry{std::move(v), {}, false}; }
    void set_str(const std::string& name, const std::string& v) { entries[name] = Entry{{}, v, true}; }
    const Entry* find_entry(const std::string& name) const {
        auto it = entries.find(name);
        return it == entries.end() ? nullptr : &it->second;
    }
    // lookup as the compiled sources write it: `auto it = prop.find(name); it != prop.end(); *it`
    struct ConstIter {
        std::map<std::string, Entry>::const_iterator it;
        const Entry& operator*() const { return it->second; }
        bool operator==(const ConstIter& o) const { return it == o.it; }
        bool operator!=(const ConstIter& o) const { return it != o.it; }
    };
    ConstIter find(const std::string& name) const { return {entries.find(name)}; }
    ConstIter end() const { return {entries.end()}; }
};

class Component {
public:
    using ComponentVisitor = std::function<void(Component*& p, bool weak)>;
    virtual ~Component() = default;
    virtual void construct(const Json& prop) { (void)prop; }
    virtual Component* underlying(const std::string& name) const { (void)name; return nullptr; }
    virtual void foreach_underlying(const ComponentVisitor& visitor) { (void)visitor; }
    virtual Json underlying_value(const std::string& query = "") const { (void)query; return {}; }
};

LM_NAMESPACE_BEGIN(comp)
template <typename T> void visit(const Component::ComponentVisitor& visitor, T*& p) {
    Component* c = p;
    visitor(c, true);
    p = dynamic_cast<T*>(c);
}
LM_NAMESPACE_END(comp)

LM_NAMESPACE_BEGIN(exception)
struct ScopedDisableFPEx {};
LM_NAMESPACE_END(exception)

enum class Error {
    None,
    Unsupported,
    Uninitialized,
    InvalidArgument,
    Unimplemented,
    IOError,
    FailedToRender,
};

LM_NAMESPACE_BEGIN(refshim)
using Factory = std::function<Component*()>;
inline std::map<std::string, Factory>& registry() {
    static std::map<std::string, Factory> r;
    return r;
}
inline Component* create(const std::string& key) {
    auto it = registry().find(key);
    return it == registry().end() ? nullptr : it->second();
}
template <typename Impl> struct Registrar {
    explicit Registrar(const char* key) { registry()[key] = [] { return static_cast<Component*>(new Impl()); }; }
};
// Components that properties refer to by locator (e.g. an area light's mesh).
inline std::map<std::string, Component*>& named() {
    static std::map<std::string, Component*> r;
    return r;
}
inline void add_named(const std::string& loc, Component* c) { named()[loc] = c; }
LM_NAMESPACE_END(refshim)

LM_NAMESPACE_BEGIN(json)
LM_NAMESPACE_BEGIN(detail)
template <typename T> struct From;
template <> struct From<double> {
    static double get(const Json::Entry& e) { return e.nums.at(0); }
};
template <> struct From<float> {
    static float get(const Json::Entry& e) { return float(e.nums.at(0)); }
};
template <> struct From<int> {
    static int get(const Json::Entry& e) { return int(e.nums.at(0)); }
};
template <> struct From<bool> {
    static bool get(const Json::Entry& e) { return e.nums.at(0) != 0; }
};
template <> struct From<Vec2> {
    static Vec2 get(const Json::Entry& e) { return Vec2(e.nums.at(0), e.nums.at(1)); }
};
template <> struct From<Vec3> {
    static Vec3 get(const Json::Entry& e) { return Vec3(e.nums.at(0), e.nums.at(1), e.nums.at(2)); }
};
template <> struct From<std::string> {
    static std::string get(const Json::Entry& e) { return e.str; }
};
LM_NAMESPACE_END(detail)

template <typename T> T value(const Json& j, const std::string& name) {
    const auto* e = j.find_entry(name);
    if (!e) throw std::invalid_argument("missing property " + name);
    return detail::From<T>::get(*e);
}
template <typename T> T value(const Json& j, const std::string& name, T&& def) {
    const auto* e = j.find_entry(name);
    return e ? detail::From<std::decay_t<T>>::get(*e) : def;
}
template <typename T> T* comp_ref_or_nullptr(const Json& j, const std::string& name) {
    const auto* e = j.find_entry(name);
    if (!e) return nullptr;
    auto it = refshim::named().find(e->str);
    return it == refshim::named().end() ? nullptr : dynamic_cast<T*>(it->second);
}
template <typename T> T* comp_ref(const Json& j, const std::string& name) {
    T* p = comp_ref_or_nullptr<T>(j, name);
    if (!p) throw std::invalid_argument("missing component reference " + name);
    return p;
}
LM_NAMESPACE_END(json)

LM_NAMESPACE_END(LM_NAMESPACE)

#define LM_COMP_REG_IMPL(ImplT, key) \
    static const LM_NAMESPACE::refshim::Registrar<ImplT> LM_TOKENPASTE2(lmref_registrar_, __LINE__){key}
#define LM_SERIALIZE_IMPL(ar) template <typename Archive> void lmref_serialize_(Archive& ar)
#define LM_INFO(...) ((void)0)
#define LM_THROW_EXCEPTION_DEFAULT(err) throw std::runtime_error("lm error: " #err)
