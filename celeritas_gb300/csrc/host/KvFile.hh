// Reader for the key/value physics input file: one record per line,
// "key count v0 v1 ...", floating point values written to round-trip.
#pragma once

#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace gbx
{
class KvFile
{
  public:
    explicit KvFile(std::string const& path)
    {
        std::ifstream in(path);
        if (!in)
        {
            throw std::runtime_error("cannot open physics file '" + path + "'");
        }
        std::string line;
        while (std::getline(in, line))
        {
            std::istringstream ss(line);
            std::string key;
            std::size_t n = 0;
            if (!(ss >> key >> n))
                continue;
            std::vector<std::string> vals(n);
            for (auto& v : vals)
                ss >> v;
            records_[key] = std::move(vals);
        }
    }

    bool has(std::string const& k) const { return records_.count(k) > 0; }

    std::vector<std::string> const& get(std::string const& k) const
    {
        auto it = records_.find(k);
        if (it == records_.end())
            throw std::runtime_error("physics file is missing key '" + k + "'");
        return it->second;
    }
    std::vector<double> dbl(std::string const& k) const
    {
        std::vector<double> r;
        for (auto const& s : this->get(k))
            r.push_back(std::strtod(s.c_str(), nullptr));
        return r;
    }
    double d(std::string const& k) const { return this->dbl(k).at(0); }
    long i(std::string const& k) const { return std::stol(this->get(k).at(0)); }
    std::string s(std::string const& k) const { return this->get(k).at(0); }

  private:
    std::map<std::string, std::vector<std::string>> records_;
};
}  // namespace gbx
