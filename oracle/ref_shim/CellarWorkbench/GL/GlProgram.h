// Stand-in for the reference's GLSL program wrapper (CellarWorkbench, not in
// this tree).  Every method aborts if called: the checker never selects a
// GLSL implementation.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <string>
#include <vector>

#include <GL3/gl3w.h>

namespace cellar {
struct GlProgramBinary
{
    GLint length = 0;
    GLenum format = 0;
    char* binary = nullptr;
};
class GlProgram
{
public:
    GlProgram() {}
    template <class... A> void reset(A...) {}
    bool addShader(GLenum, const std::vector<std::string>&) { gm_ref_gl_called("GlProgram::addShader"); }
    bool addShader(GLenum, const std::string&) { gm_ref_gl_called("GlProgram::addShader"); }
    template <class... A> bool link(A&&...) { gm_ref_gl_called("GlProgram::link"); }
    template <class... A> void pushProgram(A&&...) const { gm_ref_gl_called("GlProgram::pushProgram"); }
    template <class... A> void popProgram(A&&...) const { gm_ref_gl_called("GlProgram::popProgram"); }
    template <class... A> bool setFloat(A&&...) const { gm_ref_gl_called("GlProgram::setFloat"); }
    template <class... A> bool setInt(A&&...) const { gm_ref_gl_called("GlProgram::setInt"); }
    template <class... A> bool setVec3f(A&&...) const { gm_ref_gl_called("GlProgram::setVec3f"); }
    template <class... A> bool setVec4f(A&&...) const { gm_ref_gl_called("GlProgram::setVec4f"); }
    template <class... A> bool setMat3f(A&&...) const { gm_ref_gl_called("GlProgram::setMat3f"); }
    template <class... A> bool setMat4f(A&&...) const { gm_ref_gl_called("GlProgram::setMat4f"); }
    template <class... A> bool setSubroutine(A&&...) const { gm_ref_gl_called("GlProgram::setSubroutine"); }
    GLuint id() const { gm_ref_gl_called("GlProgram::id"); }
};
}  // namespace cellar
