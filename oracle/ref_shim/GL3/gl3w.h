// Stand-in for the OpenGL loader the reference includes.  The checker only
// runs the reference's Serial / Thread implementations; every GL entry point
// aborts if called, except the buffer create / delete and texture delete
// calls that object constructors and destructors make.  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

typedef unsigned int GLuint;
typedef int GLint;
typedef float GLfloat;
typedef unsigned int GLenum;
typedef int GLsizei;
typedef unsigned int GLbitfield;
typedef std::ptrdiff_t GLsizeiptr;
typedef std::ptrdiff_t GLintptr;

#define GL_SHADER_STORAGE_BUFFER 0x90D2
#define GL_COMPUTE_SHADER 0x91B9
#define GL_ALL_BARRIER_BITS 0xFFFFFFFF
#define GL_SHADER_STORAGE_BARRIER_BIT 0x2000
#define GL_STREAM_COPY 0x88E2
#define GL_STATIC_COPY 0x88E6
#define GL_DYNAMIC_COPY 0x88EA
#define GL_STATIC_DRAW 0x88E4
#define GL_DYNAMIC_DRAW 0x88E8
#define GL_DYNAMIC_READ 0x88E9
#define GL_MAP_READ_BIT 0x0001
#define GL_MAP_WRITE_BIT 0x0002
#define GL_MAP_INVALIDATE_RANGE_BIT 0x0004
#define GL_ACTIVE_SUBROUTINE_UNIFORM_LOCATIONS 0x8E47
#define GL_ARRAY_BUFFER 0x8892
#define GL_ELEMENT_ARRAY_BUFFER 0x8893
#define GL_FLOAT 0x1406
#define GL_UNSIGNED_INT 0x1405
#define GL_TEXTURE0 0x84C0
#define GL_TEXTURE1 0x84C1
#define GL_TEXTURE_3D 0x806F
#define GL_RGB 0x1907
#define GL_RGB32F 0x8815
#define GL_LINEAR 0x2601
#define GL_TEXTURE_MIN_FILTER 0x2801
#define GL_TEXTURE_MAG_FILTER 0x2800
#define GL_TEXTURE_WRAP_S 0x2802
#define GL_TEXTURE_WRAP_T 0x2803
#define GL_TEXTURE_WRAP_R 0x8072
#define GL_CLAMP_TO_EDGE 0x812F
#define GL_FALSE 0
#define GL_TRUE 1

[[noreturn]] inline void gm_ref_gl_called(const char* f)
{
    std::fprintf(stderr, "checker build: the graphics path (%s) is not available\n", f);
    std::abort();
}
inline void glGenBuffers(GLsizei n, GLuint* b) { for (GLsizei i = 0; i < n; ++i) b[i] = 0; }
inline void glDeleteBuffers(GLsizei, const GLuint*) {}
inline void glDeleteTextures(GLsizei, const GLuint*) {}
template <class... A> inline void glBindBuffer(A...) { gm_ref_gl_called("glBindBuffer"); }
template <class... A> inline void glBufferData(A...) { gm_ref_gl_called("glBufferData"); }
template <class... A> inline void glBufferSubData(A...) { gm_ref_gl_called("glBufferSubData"); }
template <class... A> inline void glGetBufferSubData(A...) { gm_ref_gl_called("glGetBufferSubData"); }
template <class... A> inline void glBindBufferBase(A...) { gm_ref_gl_called("glBindBufferBase"); }
template <class... A> inline void glMemoryBarrier(A...) { gm_ref_gl_called("glMemoryBarrier"); }
template <class... A> inline void* glMapBufferRange(A...) { gm_ref_gl_called("glMapBufferRange"); }
template <class... A> inline GLint glUnmapBuffer(A...) { gm_ref_gl_called("glUnmapBuffer"); }
template <class... A> inline void glDispatchCompute(A...) { gm_ref_gl_called("glDispatchCompute"); }
template <class... A> inline void glDispatchComputeGroupSizeARB(A...) { gm_ref_gl_called("glDispatchComputeGroupSizeARB"); }
template <class... A> inline GLint glGetUniformLocation(A...) { gm_ref_gl_called("glGetUniformLocation"); }
template <class... A> inline void glUniform1f(A...) { gm_ref_gl_called("glUniform1f"); }
template <class... A> inline void glUniform1i(A...) { gm_ref_gl_called("glUniform1i"); }
template <class... A> inline void glFinish(A...) { gm_ref_gl_called("glFinish"); }
template <class... A> inline void glGenTextures(A...) { gm_ref_gl_called("glGenTextures"); }
template <class... A> inline void glActiveTexture(A...) { gm_ref_gl_called("glActiveTexture"); }
template <class... A> inline void glBindTexture(A...) { gm_ref_gl_called("glBindTexture"); }
template <class... A> inline void glTexImage3D(A...) { gm_ref_gl_called("glTexImage3D"); }
template <class... A> inline void glTexParameteri(A...) { gm_ref_gl_called("glTexParameteri"); }
