// Stand-in for the reference's logging dependency (CellarWorkbench, not in
// this tree): messages are dropped unless GM_REF_LOG is set.  TEST
// INFRASTRUCTURE ONLY.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include <set>
#include <map>
#include <list>
#include <memory>
#include <functional>

namespace cellar {
struct Message
{
    char type;
    std::string text;
    Message(char t, bool, const std::string& msg, const std::string& src) : type(t), text(src + ": " + msg) {}
};
struct Log
{
    void postMessage(Message* m)
    {
        if (std::getenv("GM_REF_LOG")) std::fprintf(stderr, "[%c] %s\n", m->type, m->text.c_str());
        delete m;
    }
};
inline Log& getLog()
{
    static Log log;
    return log;
}
}  // namespace cellar
