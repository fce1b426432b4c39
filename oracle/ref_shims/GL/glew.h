/* Headless stand-in for the GL entry points the reference touches.  The
 * reference only loads matrices and sets blend/clear state; none of it feeds
 * the numbers, so every call is a no-op here.  Oracle build only. */
#ifndef WAP_REF_SHIM_GLEW_H
#define WAP_REF_SHIM_GLEW_H
typedef unsigned int GLenum;
typedef float GLfloat;
typedef double GLclampd;
typedef float GLclampf;
typedef int GLint;
typedef int GLsizei;
typedef unsigned int GLbitfield;
#define GL_PROJECTION 0x1701
#define GL_MODELVIEW 0x1700
#define GL_COLOR_BUFFER_BIT 0x4000
#define GL_DEPTH_BUFFER_BIT 0x0100
#define GL_BLEND 0x0BE2
#define GL_ONE 1
#define GL_ONE_MINUS_SRC_ALPHA 0x0303
static inline void glMatrixMode(GLenum) {}
static inline void glLoadMatrixf(const GLfloat *) {}
static inline void glClearColor(GLclampf, GLclampf, GLclampf, GLclampf) {}
static inline void glClearDepth(GLclampd) {}
static inline void glClear(GLbitfield) {}
static inline void glEnable(GLenum) {}
static inline void glBlendFunc(GLenum, GLenum) {}
static inline void glViewport(GLint, GLint, GLsizei, GLsizei) {}
static inline void glWindowPos2i(GLint, GLint) {}
static inline int glewInit() { return 0; }
#endif
