// Minimal stand-in for yaml-cpp used when compiling the reference sources.
//
// TEST INFRASTRUCTURE ONLY. It understands the flat configuration files the reference
// ships (path_tracer/config/*.yaml): one "key: value" per line, '#' comments, scalar
// values and inline sequences "[a, b, c]". That is enough for the reference's own
// parse_render_config (path_tracer/core/config.h:51-201) to run unchanged.
#pragma once

#include <cstdlib>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace YAML {

class Node {
public:
    enum class Kind { Undefined, Scalar, Sequence, Map };

    Node() = default;

    static Node scalar(const std::string& s) { Node n; n.kind_ = Kind::Scalar; n.text_ = s; return n; }
    static Node sequence(const std::vector<std::string>& items) {
        Node n; n.kind_ = Kind::Sequence;
        for (const auto& it : items) n.items_.push_back(scalar(it));
        return n;
    }
    static Node map() { Node n; n.kind_ = Kind::Map; return n; }

    bool IsMap() const { return kind_ == Kind::Map; }
    bool IsDefined() const { return kind_ != Kind::Undefined; }
    explicit operator bool() const { return IsDefined(); }

    Node operator[](const std::string& key) const {
        for (const auto& e : entries_) if (e.first.text_ == key) return e.second;
        return Node();
    }

    // Mutable lookup inserts a missing key (yaml-cpp semantics), so `node["k"] = v` works.
    Node& operator[](const std::string& key) {
        for (auto& e : entries_) if (e.first.text_ == key) return e.second;
        if (kind_ == Kind::Undefined) kind_ = Kind::Map;
        entries_.push_back({scalar(key), Node()});
        return entries_.back().second;
    }
    Node& operator=(int v) { *this = scalar(std::to_string(v)); return *this; }
    Node& operator=(float v) { std::ostringstream o; o << v; *this = scalar(o.str()); return *this; }
    Node& operator=(const std::string& v) { *this = scalar(v); return *this; }
    Node& operator=(const Node&) = default;

    void set(const std::string& key, const Node& value) { entries_.push_back({scalar(key), value}); }

    template <typename T>
    T as() const { return convert(static_cast<T*>(nullptr)); }

    using Entry = std::pair<Node, Node>;
    std::vector<Entry>::const_iterator begin() const { return entries_.begin(); }
    std::vector<Entry>::const_iterator end() const { return entries_.end(); }

private:
    void need_scalar() const {
        if (kind_ != Kind::Scalar) throw std::runtime_error("yaml shim: expected a scalar");
    }
    int convert(int*) const {
        need_scalar();
        std::size_t pos = 0;
        const int v = std::stoi(text_, &pos);
        if (pos != text_.size()) throw std::runtime_error("yaml shim: bad int '" + text_ + "'");
        return v;
    }
    float convert(float*) const {
        need_scalar();
        std::size_t pos = 0;
        const float v = std::stof(text_, &pos);
        if (pos != text_.size()) throw std::runtime_error("yaml shim: bad float '" + text_ + "'");
        return v;
    }
    bool convert(bool*) const {
        need_scalar();
        if (text_ == "true" || text_ == "True" || text_ == "yes" || text_ == "on") return true;
        if (text_ == "false" || text_ == "False" || text_ == "no" || text_ == "off") return false;
        throw std::runtime_error("yaml shim: bad bool '" + text_ + "'");
    }
    std::string convert(std::string*) const { need_scalar(); return text_; }
    std::vector<float> convert(std::vector<float>*) const {
        if (kind_ != Kind::Sequence) throw std::runtime_error("yaml shim: expected a sequence");
        std::vector<float> out;
        for (const auto& it : items_) out.push_back(it.as<float>());
        return out;
    }

    Kind kind_ = Kind::Undefined;
    std::string text_;
    std::vector<Node> items_;
    std::vector<Entry> entries_;
};

namespace shim {
inline std::string trim(const std::string& s) {
    const auto b = s.find_first_not_of(" \t\r\n");
    if (b == std::string::npos) return std::string();
    const auto e = s.find_last_not_of(" \t\r\n");
    return s.substr(b, e - b + 1);
}
inline std::string unquote(const std::string& s) {
    if (s.size() >= 2 && ((s.front() == '"' && s.back() == '"') || (s.front() == '\'' && s.back() == '\'')))
        return s.substr(1, s.size() - 2);
    return s;
}
}  // namespace shim

inline Node Load(const std::string& text) {
    Node root = Node::map();
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
        const auto hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        line = shim::trim(line);
        if (line.empty()) continue;
        const auto colon = line.find(':');
        if (colon == std::string::npos) throw std::runtime_error("yaml shim: expected 'key: value'");
        const std::string key = shim::trim(line.substr(0, colon));
        const std::string value = shim::trim(line.substr(colon + 1));
        if (!value.empty() && value.front() == '[') {
            if (value.back() != ']') throw std::runtime_error("yaml shim: unterminated sequence");
            std::vector<std::string> items;
            std::istringstream seq(value.substr(1, value.size() - 2));
            std::string item;
            while (std::getline(seq, item, ',')) {
                item = shim::trim(item);
                if (!item.empty()) items.push_back(shim::unquote(item));
            }
            root.set(key, Node::sequence(items));
        } else if (value.empty()) {
            // Nested maps are not part of the flat render configuration; keep the key
            // so strict key checking still sees it.
            root.set(key, Node::map());
        } else {
            root.set(key, Node::scalar(shim::unquote(value)));
        }
    }
    return root;
}

inline Node LoadFile(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("yaml shim: cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return Load(ss.str());
}

}  // namespace YAML
