/* Declaration-only stand-in for <GL/glew.h>.  The reference's simulation.hpp
 * reaches texture.hpp through components.hpp; no GL call is ever made by the
 * code compiled into the test oracle, so these are inert no-ops.  There is no
 * graphics stack on this machine. */
#pragma once
typedef unsigned int GLuint;
typedef unsigned int GLenum;
typedef int GLint;
typedef int GLsizei;
typedef float GLfloat;
#define GL_NO_ERROR 0
#define GL_TEXTURE_2D 0x0DE1
#define GL_SRGB8_ALPHA8 0x8C43
#define GL_RGBA 0x1908
#define GL_UNSIGNED_BYTE 0x1401
static inline GLenum glGetError(void) { return GL_NO_ERROR; }
static inline void glGenTextures(GLsizei, GLuint *) {}
static inline void glBindTexture(GLenum, GLuint) {}
static inline void glTexStorage2D(GLenum, GLsizei, GLenum, GLsizei, GLsizei) {}
static inline void glTexSubImage2D(GLenum, GLint, GLint, GLint, GLsizei, GLsizei, GLenum, GLenum,
                                   const void *) {}
static inline void glGenerateMipmap(GLenum) {}
