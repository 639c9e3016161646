/* parse(vm, search) and parse_json(vm, config, search) of include/compat/singlepulse.h over
 * small stand-ins for the variables-map and JSON types the reference uses (the program's
 * options and a two-entry ddplan configuration): prints every row's fields, the command-line
 * rows first, so the test can check them.  argv[1], when given, is a ddplan file.  No GPU call
 * is made: parsing only configures SinglePulse objects. */
#include <cstdio>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "compat/singlepulse.h"

unsigned int dbscan_radius = 4;
unsigned int dbscan_k = 2;
unsigned int num_threads = 1;
bool repeater = false;
bool dumptim = false;

struct OptionValue {
    std::string s;
    template <class T> T as() const
    {
        std::istringstream in(s);
        T v{};
        in >> v;
        return v;
    }
};
template <> std::string OptionValue::as<std::string>() const { return s; }
template <> std::vector<float> OptionValue::as<std::vector<float>>() const
{
    std::istringstream in(s);
    std::vector<float> v;
    for (float x; in >> x;) v.push_back(x);
    return v;
}
template <> std::vector<std::string> OptionValue::as<std::vector<std::string>>() const
{
    std::istringstream in(s);
    std::vector<std::string> v;
    for (std::string x; in >> x;) v.push_back(x);
    return v;
}
struct VariablesMap {
    std::map<std::string, std::string> m;
    OptionValue operator[](const char *k) const
    {
        auto it = m.find(k);
        return {it == m.end() ? std::string() : it->second};
    }
    size_t count(const char *k) const { return m.count(k); }
};

/* a JSON value: number, string, object or array */
struct Json {
    double num = 0.;
    std::string str;
    std::map<std::string, Json> obj;
    std::vector<Json> arr;
    Json() = default;
    Json(double v) : num(v) {}
    Json(const char *v) : str(v) {}
    Json(std::initializer_list<std::pair<const std::string, Json>> o) : obj(o) {}
    static Json array(std::vector<Json> a)
    {
        Json j;
        j.arr = std::move(a);
        return j;
    }
    Json operator[](const char *k) const
    {
        auto it = obj.find(k);
        return it == obj.end() ? Json() : it->second;
    }
    operator int() const { return (int)num; }
    operator long() const { return (long)num; }
    operator float() const { return (float)num; }
    operator double() const { return num; }
    operator bool() const { return num != 0.; }
    operator std::string() const { return str; }
    std::vector<Json>::const_iterator begin() const { return arr.begin(); }
    std::vector<Json>::const_iterator end() const { return arr.end(); }
    const Json &front() const { return arr.front(); }
    const Json &back() const { return arr.back(); }
};

static void print(const std::vector<SinglePulse> &rows)
{
    for (const auto &r : rows) {
        std::printf("row %d td %d fd %d dms %g ddm %g ndm %ld snrloss %g maxw %g bswidth %g thre %g "
                    "radius %g minpts %d iqr %d nzap %zu rfi", r.id, r.td, r.fd, r.dms, r.ddm, r.ndm,
                    r.snrloss, r.maxw, r.bswidth, r.thre, r.radius_smearing, r.minpts, (int)r.iqr,
                    r.zaplist.size());
        for (const auto &op : r.rfilist)
            for (const auto &w : op) std::printf(" %s", w.c_str());
        std::printf("\n");
    }
}

int main(int argc, char **argv)
{
    VariablesMap vm;
    vm.m = {{"baseline", "0 0.1"}, {"fill", "mean"}, {"bandlimit", "10"}, {"bandlimitKT", "10"},
            {"widthlimit", "0.01"}, {"threMask", "10"}, {"threKadaneF", "7"},
            {"threKadaneT", "7"}, {"dms", "0"}, {"ddm", "1"}, {"ndm", "1000"}, {"overlap", "0"},
            {"minw", "0.0001"}, {"snrloss", "0.1"}, {"maxw", "0.02"}, {"thre", "7"},
            {"radius", "1"}, {"neighbors", "2"}, {"maxncand", "100"}, {"minpts", "5"},
            {"mean", "0"}, {"std", "0"}, {"nbits", "8"}, {"format", "sigproc"},
            {"rfi", "zdot kadaneF 8 4 zap 1100 1200"}};
    if (argc > 1) vm.m["ddplan"] = argv[1];
    std::vector<SinglePulse> search;
    parse(vm, search);
    print(search);

    Json row = {{"downsample", {{"td", 2.}, {"fd", 1.}}},
                {"baseline", {{"width", 0.2}}},
                {"subdedispersion", {{"dms", 500.}, {"ddm", 0.2}, {"ndm", 5000.}, {"overlap", 0.}}},
                {"rfi", {{"bandlimit", 10.}, {"bandlimitKT", 10.}, {"widthlimit", 0.02},
                         {"threMask", 10.}, {"threKadaneF", 8.}, {"threKadaneT", 7.}}},
                {"boxcar", {{"minw", 0.0001}, {"snrloss", 0.1}, {"maxw", 0.05}, {"iqr", 1.}}},
                {"clustering", {{"thre", 6.5}, {"radius", 2.}, {"neighbors", 2.}, {"maxncand", 50.},
                                {"minpts", 3.}, {"drop", 0.}}}};
    row.obj["rfi"].obj["zaplist"] = Json::array({Json::array({Json(1100.), Json(1200.)})});
    row.obj["rfi"].obj["rfilist"] = Json::array({Json::array({Json("kadaneF"), Json("8"), Json("4")}),
                                                 Json::array({Json("zdot")})});
    Json row2 = row;
    row2.obj["downsample"].obj["td"] = 4.;
    row2.obj["subdedispersion"].obj["dms"] = 1500.;
    row2.obj["rfi"].obj["zaplist"] = Json::array({Json::array({Json(1300.), Json(1310.)})});
    row2.obj["rfi"].obj["rfilist"] = Json::array({Json::array({Json("zap"), Json("1"), Json("2")}),
                                                  Json::array({Json("zero")})});
    Json config;
    config.obj["ddplan"] = Json::array({row, row2});
    std::vector<SinglePulse> search2;
    parse_json(vm, config, search2);
    print(search2);
    return 0;
}
