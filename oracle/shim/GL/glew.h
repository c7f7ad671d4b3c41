// Test infrastructure: no-op OpenGL entry points so that the reference's render code
// (code/nans.cpp:1766-2025, code/utilities.cpp:1-23) compiles in a headless oracle build.
// Nothing here draws; physics never calls these.
#ifndef NANS_SHIM_GLEW_H
#define NANS_SHIM_GLEW_H

typedef unsigned int GLenum;
typedef unsigned int GLuint;
typedef int GLint;
typedef int GLsizei;
typedef float GLfloat;
typedef unsigned char GLboolean;

#define GL_FALSE 0
#define GL_TRIANGLES 0x0004
#define GL_UNSIGNED_INT 0x1405
#define GL_TEXTURE_2D 0x0DE1
#define GL_TEXTURE0 0x84C0
#define GL_TEXTURE1 0x84C1
#define GL_FRONT_AND_BACK 0x0408
#define GL_LINE 0x1B01
#define GL_FILL 0x1B02

static inline void glUseProgram(GLuint) {}
static inline GLint glGetUniformLocation(GLuint, const char *) { return -1; }
static inline void glUniform1f(GLint, GLfloat) {}
static inline void glUniform1i(GLint, GLint) {}
static inline void glUniform3f(GLint, GLfloat, GLfloat, GLfloat) {}
static inline void glUniform3fv(GLint, GLsizei, const GLfloat *) {}
static inline void glUniformMatrix4fv(GLint, GLsizei, GLboolean, const GLfloat *) {}
static inline void glBindVertexArray(GLuint) {}
static inline void glBindTexture(GLenum, GLuint) {}
static inline void glActiveTexture(GLenum) {}
static inline void glDrawArrays(GLenum, GLint, GLsizei) {}
static inline void glDrawElements(GLenum, GLsizei, GLenum, const void *) {}
static inline void glPolygonMode(GLenum, GLenum) {}

#endif
