// Compile-only stand-in for the nlohmann JSON header, used when building the
// reference's host stepping loop as a CPU oracle. The oracle never reads or
// writes JSON: this class accepts the calls that the reference's diagnostic
// output code makes and does nothing; parsing and value extraction throw.
// It is NOT the nlohmann library.
#pragma once

#include <cstddef>
#include <initializer_list>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace nlohmann
{
template<class T, class = void>
struct adl_serializer;

class json
{
  public:
    using size_type = std::size_t;
    using value_type = json;

    class iterator
    {
      public:
        json& operator*() const { return *j_; }
        json* operator->() const { return j_; }
        iterator& operator++() { return *this; }
        bool operator==(iterator const&) const { return true; }
        bool operator!=(iterator const&) const { return false; }
        std::string key() const { return {}; }
        json& value() const { return *j_; }
        json* j_{nullptr};
    };
    using const_iterator = iterator;

    struct items_proxy
    {
        iterator begin() const { return {}; }
        iterator end() const { return {}; }
    };

    json() = default;
    json(json const&) = default;
    json(json&&) = default;
    json& operator=(json const&) = default;
    json& operator=(json&&) = default;
    json(std::nullptr_t) {}
    json(std::initializer_list<json>) {}
    template<class T>
    json(T const&)
    {
    }

    template<class T>
    json& operator=(T const&)
    {
        return *this;
    }

    static json array(std::initializer_list<json> = {}) { return {}; }
    static json object(std::initializer_list<json> = {}) { return {}; }
    template<class... Args>
    static json parse(Args&&...)
    {
        throw std::runtime_error("JSON parsing is unavailable in the oracle");
    }

    template<class K>
    json& operator[](K const&)
    {
        return *this;
    }
    template<class K>
    json const& operator[](K const&) const
    {
        return *this;
    }
    template<class K>
    json& at(K const&)
    {
        throw std::out_of_range("JSON is unavailable in the oracle");
    }
    template<class K>
    json const& at(K const&) const
    {
        throw std::out_of_range("JSON is unavailable in the oracle");
    }
    template<class K>
    iterator find(K const&) const
    {
        return {};
    }
    template<class K>
    bool contains(K const&) const
    {
        return false;
    }
    template<class K>
    size_type count(K const&) const
    {
        return 0;
    }
    iterator begin() const { return {}; }
    iterator end() const { return {}; }
    items_proxy items() const { return {}; }
    size_type size() const { return 0; }
    bool empty() const { return true; }
    bool is_null() const { return true; }
    bool is_object() const { return false; }
    bool is_array() const { return false; }
    bool is_string() const { return false; }
    bool is_number() const { return false; }
    bool is_boolean() const { return false; }
    template<class... Args>
    std::string dump(Args&&...) const
    {
        return "null";
    }
    template<class T>
    void push_back(T const&)
    {
    }
    void push_back(std::initializer_list<json>) {}
    std::string key() const { return {}; }
    json value() const { return {}; }
    template<class... Args>
    json& emplace_back(Args&&...)
    {
        return *this;
    }
    json& back() { return *this; }
    json const& back() const { return *this; }
    template<class T>
    T get() const
    {
        throw std::runtime_error("JSON is unavailable in the oracle");
    }
    template<class T>
    T& get_to(T& v) const
    {
        throw std::runtime_error("JSON is unavailable in the oracle");
        return v;
    }
    template<class T>
    operator T() const
    {
        throw std::runtime_error("JSON is unavailable in the oracle");
    }
    template<class T>
    bool operator==(T const&) const
    {
        return false;
    }
    template<class T>
    bool operator!=(T const&) const
    {
        return true;
    }
};

inline std::ostream& operator<<(std::ostream& os, json const&)
{
    return os;
}

}  // namespace nlohmann
