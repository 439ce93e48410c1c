/*---------------------------------------------------------------------------*\
  harness_io.H - the record files the oracle harnesses read and write.

  Test infrastructure only.  Record file: "CFXREC1\n", then records of
    char name[32]; char dtype[8] ("i4"|"f8"|"s"); int64 count; data
\*---------------------------------------------------------------------------*/

#ifndef cfx_harness_io_H
#define cfx_harness_io_H

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace
{

using namespace Foam;

struct Rec
{
    std::string dtype;
    std::vector<char> data;
    int64_t count = 0;
};

typedef std::map<std::string, Rec> RecMap;

RecMap readRecs(const char* path)
{
    RecMap m;
    FILE* fh = std::fopen(path, "rb");
    if (!fh) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
    char magic[8];
    if (std::fread(magic, 1, 8, fh) != 8 || std::memcmp(magic, "CFXREC1\n", 8))
    {
        std::fprintf(stderr, "bad record file\n"); std::exit(2);
    }
    while (true)
    {
        char name[33] = {0}, dt[9] = {0};
        int64_t n;
        if (std::fread(name, 1, 32, fh) != 32) break;
        if (std::fread(dt, 1, 8, fh) != 8) break;
        if (std::fread(&n, 8, 1, fh) != 1) break;
        Rec r;
        r.dtype = dt;
        r.count = n;
        size_t es = r.dtype == "f8" ? 8 : r.dtype == "i4" ? 4 : 1;
        r.data.resize(es*n);
        if (n && std::fread(r.data.data(), es, n, fh) != size_t(n)) break;
        m[name] = r;
    }
    std::fclose(fh);
    return m;
}

struct Writer
{
    FILE* fh;
    explicit Writer(const char* path) : fh(std::fopen(path, "wb"))
    {
        std::fwrite("CFXREC1\n", 1, 8, fh);
    }
    ~Writer() { std::fclose(fh); }
    void put(const std::string& name, const char* dt, const void* p, int64_t n, size_t es)
    {
        char nm[32] = {0}, d[8] = {0};
        std::strncpy(nm, name.c_str(), 31);
        std::strncpy(d, dt, 7);
        std::fwrite(nm, 1, 32, fh);
        std::fwrite(d, 1, 8, fh);
        std::fwrite(&n, 8, 1, fh);
        if (n) std::fwrite(p, es, n, fh);
    }
    void f8(const std::string& name, const scalarUList& v) { put(name, "f8", v.cdata(), v.size(), 8); }
    void f8(const std::string& name, double v) { put(name, "f8", &v, 1, 8); }
    void i4(const std::string& name, const labelUList& v) { put(name, "i4", v.cdata(), v.size(), 4); }
    void i4(const std::string& name, int v) { put(name, "i4", &v, 1, 4); }
    void vec(const std::string& name, const vectorField& v)
    {
        put(name, "f8", v.cdata(), 3*v.size(), 8);
    }
};

labelList getL(const RecMap& m, const char* k)
{
    const Rec& r = m.at(k);
    labelList out(r.count);
    std::memcpy(out.data(), r.data.data(), 4*r.count);
    return out;
}

scalarField getF(const RecMap& m, const char* k)
{
    const Rec& r = m.at(k);
    scalarField out(r.count);
    std::memcpy(out.data(), r.data.data(), 8*r.count);
    return out;
}

std::string getS(const RecMap& m, const char* k)
{
    const Rec& r = m.at(k);
    return std::string(r.data.begin(), r.data.end());
}

bool has(const RecMap& m, const char* k) { return m.count(k) > 0; }

} // End anonymous namespace

#endif
