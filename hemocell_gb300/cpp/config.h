// Minimal XML configuration reader with the reference's access pattern:
// cfg["domain"]["dx"].read<double>() (config/config.h, config/config.cpp:70-87);
// a missing key throws std::invalid_argument as the reference does.
#pragma once

#include <array>
#include <cctype>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace hemo {

struct XMLNode {
  std::string name, text;
  std::vector<std::unique_ptr<XMLNode>> children;
  XMLNode* missing = nullptr;  // set on lookups of absent keys
  std::string path;

  XMLNode& operator[](const std::string& key) {
    for (auto& c : children)
      if (c->name == key) return *c;
    throw std::invalid_argument("(Config) key not found: " + path + "/" + key);
  }
  template <class T>
  T read() const {
    std::istringstream in(text);
    T v;
    if (!(in >> v)) throw std::invalid_argument("(Config) cannot parse value of " + path);
    return v;
  }
  // <InnerEdges><Edge> a b </Edge>...</InnerEdges> -> flat pair list
  std::vector<int> readPairs() const {
    std::vector<int> out;
    for (auto& c : children) {
      std::istringstream in(c->text);
      int a, b;
      if (!(in >> a >> b)) throw std::invalid_argument("(Config) bad pair in " + path);
      out.push_back(a);
      out.push_back(b);
    }
    return out;
  }
};

class Config {
 public:
  explicit Config(const char* path) {
    std::ifstream f(path);
    if (!f) throw std::invalid_argument(std::string("cannot open ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    src_ = ss.str();
    pos_ = 0;
    root_ = std::make_unique<XMLNode>();
    root_->name = "#document";
    parseChildren(*root_, "");
    // the document element (<hemocell>) is the lookup root
    for (auto& c : root_->children) top_ = c.get();
    if (!top_) throw std::invalid_argument(std::string("empty configuration ") + path);
  }
  XMLNode& operator[](const std::string& key) { return (*top_)[key]; }

 private:
  std::string src_;
  size_t pos_ = 0;
  std::unique_ptr<XMLNode> root_;
  XMLNode* top_ = nullptr;

  void skip(const char* end) {
    size_t e = src_.find(end, pos_);
    if (e == std::string::npos) throw std::invalid_argument("unterminated XML construct");
    pos_ = e + std::string(end).size();
  }
  void parseChildren(XMLNode& parent, const std::string& closing) {
    while (pos_ < src_.size()) {
      size_t lt = src_.find('<', pos_);
      if (lt == std::string::npos) break;
      parent.text += src_.substr(pos_, lt - pos_);
      pos_ = lt;
      if (src_.compare(pos_, 4, "<!--") == 0) { skip("-->"); continue; }
      if (src_.compare(pos_, 2, "<?") == 0) { skip("?>"); continue; }
      if (src_.compare(pos_, 2, "</") == 0) {
        size_t gt = src_.find('>', pos_);
        std::string nm = src_.substr(pos_ + 2, gt - pos_ - 2);
        while (!nm.empty() && std::isspace((unsigned char)nm.back())) nm.pop_back();
        if (nm != closing) throw std::invalid_argument("mismatched closing tag " + nm);
        pos_ = gt + 1;
        return;
      }
      size_t gt = src_.find('>', pos_);
      if (gt == std::string::npos) throw std::invalid_argument("unterminated tag");
      std::string tag = src_.substr(pos_ + 1, gt - pos_ - 1);
      bool selfclose = !tag.empty() && tag.back() == '/';
      if (selfclose) tag.pop_back();
      std::string nm = tag.substr(0, tag.find_first_of(" \t\r\n"));
      auto child = std::make_unique<XMLNode>();
      child->name = nm;
      child->path = parent.path + "/" + nm;
      pos_ = gt + 1;
      if (!selfclose) parseChildren(*child, nm);
      parent.children.push_back(std::move(child));
    }
    if (!closing.empty()) throw std::invalid_argument("missing closing tag " + closing);
  }
};

}  // namespace hemo
