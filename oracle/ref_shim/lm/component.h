// Oracle (test infrastructure only): stand-in for the reference's component framework
// (include/lm/component.h with jsontype.h, json.h, logger.h, exception.h, serial.h), which needs
// nlohmann_json and cereal. oracle/Makefile builds _ref/include/lm/ as links to the reference's
// headers, with these framework headers linked in place of the reference's own, so the
// reference's interface headers (scene.h, path.h, light.h, material.h, camera.h, film.h, mesh.h,
// ...) compile unmodified with these definitions behind their `#include "component.h"`.
//
// What the compiled sources use, with the behaviour they rely on:
//   * Json -- a small JSON value (null, number, string, array, object) with the nlohmann-style
//     access they call: operator[], size(), find() / end() / value(), get<T>() and implicit
//     conversions to numbers, strings, vectors and 4x4 matrices; brace-initialised objects;
//     raw pointers held as values (model_wavefrontobj.cpp:83-86 hands its mesh components the
//     model and a face list that way, read back with get<T*>());
//   * json::value / value_or_none / comp_ref / comp_ref_or_nullptr / merge -- property reads;
//   * Component (key, locator, name, make_loc, construct / underlying hooks), Component::Ptr;
//   * comp::create (factory by key, constructed with its properties), comp::get (a locator
//     registered with refshim::add_named, or one below it resolved through underlying(), as
//     component.cpp:322-360 walks the hierarchy), comp::visit, comp::detail::ContextInstance
//     (the singleton context objloader.cpp keeps);
//   * fmt::format with positional "{}" fields;
//   * LM_COMP_REG_IMPL -- factory registration by key;
//   * LM_SERIALIZE_IMPL -- opens a serialization template that is never instantiated;
//   * logging macros, dropped; errors thrown as std::runtime_error; the floating-point-exception
//     guard a no-op (exceptions are never enabled in this library).
#pragma once
#include <pch.h>
#include <lm/common.h>
#include <lm/math.h>

LM_NAMESPACE_BEGIN(LM_NAMESPACE)

// ------------------------------------------------------------------------------------------------
// Json

class Json {
public:
    enum class Type { Null, Number, String, Array, Object, Pointer };

    Json() = default;
    Json(std::nullptr_t) {}
    Json(double v) : type_(Type::Number), num_(v) {}
    Json(float v) : type_(Type::Number), num_(v) {}
    Json(int v) : type_(Type::Number), num_(v) {}
    Json(unsigned int v) : type_(Type::Number), num_(v) {}
    Json(long v) : type_(Type::Number), num_(double(v)) {}
    Json(long long v) : type_(Type::Number), num_(double(v)) {}
    Json(unsigned long v) : type_(Type::Number), num_(double(v)) {}
    Json(bool v) : type_(Type::Number), num_(v ? 1 : 0) {}
    Json(const char* s) : type_(Type::String), str_(s) {}
    Json(const std::string& s) : type_(Type::String), str_(s) {}
    Json(char* s) : type_(Type::String), str_(s) {}
    template <typename T> Json(T* p) : type_(Type::Pointer), ptr_(static_cast<const void*>(p)) {}
    Json(const Vec2& v) : type_(Type::Array) { arr_ = {Json(v.x), Json(v.y)}; }
    Json(const Vec3& v) : type_(Type::Array) { arr_ = {Json(v.x), Json(v.y), Json(v.z)}; }
    Json(const Vec4& v) : type_(Type::Array) { arr_ = {Json(v.x), Json(v.y), Json(v.z), Json(v.w)}; }
    Json(const Mat4& m) : type_(Type::Array) {
        for (int c = 0; c < 4; c++) arr_.push_back(Json(m[c]));
    }
    // an object from {"name", value} pairs
    struct Item {
        std::string key;
        std::shared_ptr<Json> value;
        template <typename T> Item(const char* k, const T& v) : key(k), value(std::make_shared<Json>(v)) {}
    };
    Json(std::initializer_list<Item> items) : type_(Type::Object) {
        for (const auto& it : items) obj_[it.key] = *it.value;
    }
    static Json array() { Json j; j.type_ = Type::Array; return j; }
    static Json object() { Json j; j.type_ = Type::Object; return j; }

    Type type() const { return type_; }
    bool is_null() const { return type_ == Type::Null; }
    size_t size() const { return type_ == Type::Array ? arr_.size() : type_ == Type::Object ? obj_.size() : 0; }
    void push_back(Json v) {
        type_ = Type::Array;
        arr_.push_back(std::move(v));
    }
    const Json& operator[](size_t i) const { return arr_.at(i); }
    const Json& operator[](int i) const { return arr_.at(size_t(i)); }
    const Json& operator[](const std::string& k) const {
        auto it = obj_.find(k);
        if (it == obj_.end()) throw std::out_of_range("missing property " + k);
        return it->second;
    }
    const Json& operator[](const char* k) const { return (*this)[std::string(k)]; }
    Json& operator[](const std::string& k) {
        type_ = Type::Object;
        return obj_[k];
    }
    Json& operator[](const char* k) { return (*this)[std::string(k)]; }

    struct const_iterator {
        std::map<std::string, Json>::const_iterator it;
        const Json& operator*() const { return it->second; }
        const Json* operator->() const { return &it->second; }
        const Json& value() const { return it->second; }
        const std::string& key() const { return it->first; }
        bool operator==(const const_iterator& o) const { return it == o.it; }
        bool operator!=(const const_iterator& o) const { return it != o.it; }
    };
    const_iterator find(const std::string& k) const { return {obj_.find(k)}; }
    const_iterator end() const { return {obj_.end()}; }
    bool contains(const std::string& k) const { return obj_.count(k) > 0; }
    // nlohmann's merge_patch restricted to one level: o's keys replace this object's.
    Json merged(const Json& o) const {
        Json r = *this;
        r.type_ = Type::Object;
        for (const auto& [k, v] : o.obj_) r.obj_[k] = v;
        return r;
    }
    const void* pointer() const {
        if (type_ != Type::Pointer) throw std::invalid_argument("not a pointer");
        return ptr_;
    }

    double number() const {
        if (type_ != Type::Number) throw std::invalid_argument("not a number");
        return num_;
    }
    const std::string& string() const {
        if (type_ != Type::String) throw std::invalid_argument("not a string");
        return str_;
    }
    template <typename T> T get() const;
    // nlohmann's j.value(key, default)
    template <typename T> T value(const std::string& k, const T& def) const {
        auto it = obj_.find(k);
        return it == obj_.end() ? def : it->second.template get<T>();
    }
    std::string value(const std::string& k, const char* def) const {
        auto it = obj_.find(k);
        return it == obj_.end() ? std::string(def) : it->second.string();
    }

    operator double() const { return number(); }
    operator float() const { return float(number()); }
    operator int() const { return int(number()); }
    operator unsigned int() const { return (unsigned int)(number()); }
    operator long long() const { return (long long)(number()); }
    operator bool() const { return number() != 0; }
    operator std::string() const { return string(); }
    operator Vec2() const { return Vec2((*this)[0].number(), (*this)[1].number()); }
    operator Vec3() const { return Vec3((*this)[0].number(), (*this)[1].number(), (*this)[2].number()); }
    operator Vec4() const {
        return Vec4((*this)[0].number(), (*this)[1].number(), (*this)[2].number(), (*this)[3].number());
    }
    operator Mat4() const {
        Mat4 m;
        for (int c = 0; c < 4; c++) m[c] = Vec4((*this)[c]);
        return m;
    }

private:
    Type type_ = Type::Null;
    double num_ = 0;
    std::string str_;
    std::vector<Json> arr_;
    std::map<std::string, Json> obj_;
    const void* ptr_ = nullptr;
};

template <typename T> inline T Json::get() const {
    if constexpr (std::is_pointer_v<T>) return static_cast<T>(const_cast<void*>(pointer()));
    else return static_cast<T>(*this);
}
template <> inline std::string Json::get<std::string>() const { return string(); }

// ------------------------------------------------------------------------------------------------
// Errors, logging and formatting

enum class Error {
    None,
    Unsupported,
    Uninitialized,
    InvalidArgument,
    Unimplemented,
    IOError,
    FailedToRender,
};

LM_NAMESPACE_BEGIN(exception)
struct ScopedDisableFPEx {};
LM_NAMESPACE_END(exception)

LM_NAMESPACE_END(LM_NAMESPACE)
namespace fmt {
// Each "{}" of f takes the next argument, written as operator<< writes it.
template <typename... Args> std::string format(const std::string& f, const Args&... args) {
    std::vector<std::string> parts;
    ((parts.push_back((std::ostringstream() << args).str())), ...);
    std::string out;
    size_t next = 0;
    for (size_t i = 0; i < f.size(); i++) {
        if (f[i] == '{' && i + 1 < f.size() && f[i + 1] == '}' && next < parts.size()) {
            out += parts[next++];
            i++;
        } else {
            out += f[i];
        }
    }
    return out;
}
}  // namespace fmt
LM_NAMESPACE_BEGIN(LM_NAMESPACE)

// ------------------------------------------------------------------------------------------------
// Components

class Component {
public:
    template <typename InterfaceT> using Ptr = std::unique_ptr<InterfaceT>;
    using ComponentVisitor = std::function<void(Component*& p, bool weak)>;

    virtual ~Component() = default;
    const std::string& key() const { return key_; }
    const std::string& loc() const { return loc_; }
    const std::string name() const {
        const auto i = loc_.find_last_of('.');
        return i == std::string::npos ? loc_ : loc_.substr(i + 1);
    }
    const std::string make_loc(const std::string& base, const std::string& child) const { return base + "." + child; }
    const std::string make_loc(const std::string& child) const { return make_loc(loc(), child); }

    virtual void construct(const Json& prop) { (void)prop; }
    virtual Component* underlying(const std::string& name) const { (void)name; return nullptr; }
    virtual void foreach_underlying(const ComponentVisitor& visitor) { (void)visitor; }
    virtual Json underlying_value(const std::string& query = "") const { (void)query; return {}; }
    virtual void* underlying_raw_pointer(const std::string& query = "") const { (void)query; return nullptr; }

    void lmref_set_ids(const std::string& key, const std::string& loc) {
        key_ = key;
        loc_ = loc;
    }

private:
    std::string key_;
    std::string loc_;
};

LM_NAMESPACE_BEGIN(refshim)
using Factory = std::function<Component*()>;
inline std::map<std::string, Factory>& registry() {
    static std::map<std::string, Factory> r;
    return r;
}
inline std::map<std::string, Component*>& named() {
    static std::map<std::string, Component*> r;
    return r;
}
// Makes a component registered under `key` (nullptr if none).
inline Component* make(const std::string& key) {
    auto it = registry().find(key);
    return it == registry().end() ? nullptr : it->second();
}
// Makes the factory's creations reachable by locator (comp::get, json::comp_ref).
inline void add_named(const std::string& loc, Component* c) { named()[loc] = c; }
inline void remove_named(const std::string& loc) { named().erase(loc); }
template <typename Impl> struct Registrar {
    explicit Registrar(const char* key) { registry()[key] = [] { return static_cast<Component*>(new Impl()); }; }
};
LM_NAMESPACE_END(refshim)

LM_NAMESPACE_BEGIN(comp)
// A registered locator, or one below the longest registered prefix reached through underlying()
// one dot-separated name at a time.
template <typename T> T* get(const std::string& locator) {
    const auto& n = refshim::named();
    if (const auto it = n.find(locator); it != n.end()) return dynamic_cast<T*>(it->second);
    for (size_t i = locator.rfind('.'); i != std::string::npos && i > 0; i = locator.rfind('.', i - 1)) {
        const auto it = n.find(locator.substr(0, i));
        if (it == n.end()) continue;
        Component* c = it->second;
        std::string rest = locator.substr(i + 1);
        while (c && !rest.empty()) {
            const size_t j = rest.find('.');
            c = c->underlying(rest.substr(0, j));
            rest = j == std::string::npos ? std::string() : rest.substr(j + 1);
        }
        return dynamic_cast<T*>(c);
    }
    return nullptr;
}
template <typename InterfaceT>
Component::Ptr<InterfaceT> create(const std::string& key, const std::string& loc, const Json& prop = {}) {
    std::unique_ptr<Component> c(refshim::make(key));
    if (!c) return nullptr;
    c->lmref_set_ids(key, loc);
    c->construct(prop);
    auto* p = dynamic_cast<InterfaceT*>(c.get());
    if (!p) return nullptr;
    c.release();
    return Component::Ptr<InterfaceT>(p);
}
template <typename T> void visit(const Component::ComponentVisitor& visitor, T*& p) {
    Component* c = p;
    visitor(c, true);
    p = dynamic_cast<T*>(c);
}
template <typename T> void visit(const Component::ComponentVisitor& visitor, Component::Ptr<T>& p) {
    Component* c = p.get();
    visitor(c, false);
}
LM_NAMESPACE_BEGIN(detail)
// A process-wide context component created by key (the objloader's).
template <typename ContextComponentT> class ContextInstance {
public:
    static ContextComponentT& get() {
        if (!ctx()) throw std::runtime_error("lm error: Uninitialized context component");
        return *ctx();
    }
    static void init(const std::string& type, const Json& prop) {
        ctx() = comp::create<ContextComponentT>(type, "$", prop);
        if (!ctx()) throw std::invalid_argument("no context component registered as " + type);
    }
    static void shutdown() { ctx().reset(); }
    static bool initialized() { return bool(ctx()); }

private:
    static Component::Ptr<ContextComponentT>& ctx() {
        static Component::Ptr<ContextComponentT> p;
        return p;
    }
};
LM_NAMESPACE_END(detail)
LM_NAMESPACE_END(comp)

// ------------------------------------------------------------------------------------------------
// Property reads

LM_NAMESPACE_BEGIN(json)
template <typename T> T value(const Json& j, const std::string& name) {
    const auto it = j.find(name);
    if (it == j.end()) throw std::invalid_argument("missing property " + name);
    return (*it).template get<T>();
}
template <typename T> T value(const Json& j, const std::string& name, T&& def) {
    const auto it = j.find(name);
    if (it == j.end()) return def;
    return (*it).template get<std::decay_t<T>>();
}
inline std::string value(const Json& j, const std::string& name, const char* def) {
    const auto it = j.find(name);
    return it == j.end() ? std::string(def) : (*it).get<std::string>();
}
template <typename T> std::optional<T> value_or_none(const Json& j, const std::string& name) {
    const auto it = j.find(name);
    if (it == j.end()) return {};
    return (*it).template get<T>();
}
template <typename T> T* comp_ref_or_nullptr(const Json& j, const std::string& name) {
    const auto it = j.find(name);
    if (it == j.end()) return nullptr;
    return comp::get<T>((*it).get<std::string>());
}
template <typename T> T* comp_ref(const Json& j, const std::string& name) {
    T* p = comp_ref_or_nullptr<T>(j, name);
    if (!p) throw std::invalid_argument("missing component reference " + name);
    return p;
}
inline Json merge(const Json& a, const Json& b) { return a.merged(b); }
LM_NAMESPACE_END(json)

LM_NAMESPACE_END(LM_NAMESPACE)

#define LM_COMP_REG_IMPL(ImplT, key) \
    static const LM_NAMESPACE::refshim::Registrar<ImplT> LM_TOKENPASTE2(lmref_registrar_, __LINE__){key}
#define LM_SERIALIZE_IMPL(ar) template <typename Archive> void lmref_serialize_(Archive& ar)
#define LM_INFO(...) ((void)0)
#define LM_WARN(...) ((void)0)
#define LM_ERROR(...) ((void)0)
#define LM_DEBUG(...) ((void)0)
#define LM_INDENT() ((void)0)
#define LM_THROW_EXCEPTION_DEFAULT(err) throw std::runtime_error("lm error: " #err)
#define LM_THROW_EXCEPTION(err, ...) throw std::runtime_error("lm error: " #err)
