/* Stand-in for <GL/gl.h> when the reference's kd-tree and shape sources are compiled as a
 * CPU test oracle: the intersection code never draws, so every GL entry point the preview
 * methods name is a no-op here and no graphics library is linked. */
#ifndef MILTON_REF_SHIM_GL_H_
#define MILTON_REF_SHIM_GL_H_
typedef unsigned int GLenum;
typedef unsigned int GLuint;
typedef unsigned int GLbitfield;
typedef int GLint;
typedef int GLsizei;
typedef float GLfloat;
typedef double GLdouble;
typedef float GLclampf;
typedef double GLclampd;
typedef unsigned char GLboolean;
#define GL_BLEND 0x0BE2
#define GL_COMPILE_AND_EXECUTE 0x1301
#define GL_CULL_FACE 0x0B44
#define GL_DIFFUSE 0x1201
#define GL_DOUBLE 0x140A
#define GL_ENABLE_BIT 0x00002000
#define GL_FRONT_AND_BACK 0x0408
#define GL_LIGHTING 0x0B50
#define GL_LINES 0x0001
#define GL_MODELVIEW_MATRIX 0x0BA6
#define GL_NORMAL_ARRAY 0x8075
#define GL_ONE 1
#define GL_QUADS 0x0007
#define GL_SRC_ALPHA 0x0302
#define GL_TEXTURE_COORD_ARRAY 0x8078
#define GL_TRIANGLES 0x0004
#define GL_UNSIGNED_INT 0x1405
#define GL_VERTEX_ARRAY 0x8074
#define GL_COLOR_MATERIAL 0x0B57
#define GL_AMBIENT_AND_DIFFUSE 0x1602
#define GL_ALWAYS 0x7000
#define GL_BACK 0x7001
#define GL_CCW 0x7002
#define GL_CONSTANT_ALPHA 0x7003
#define GL_CONSTANT_ATTENUATION 0x7004
#define GL_CONSTANT_COLOR 0x7005
#define GL_CW 0x7006
#define GL_DECR 0x7007
#define GL_DECR_WRAP 0x7008
#define GL_DONT_CARE 0x7009
#define GL_DST_ALPHA 0x700A
#define GL_DST_COLOR 0x700B
#define GL_EQUAL 0x700C
#define GL_EXP 0x700D
#define GL_EXP2 0x700E
#define GL_FALSE 0x700F
#define GL_FASTEST 0x7010
#define GL_FILL 0x7011
#define GL_FOG_COORD 0x7012
#define GL_FOG_COORD_ARRAY 0x7013
#define GL_FRAGMENT_DEPTH 0x7014
#define GL_FRONT 0x7015
#define GL_FUNC_ADD 0x7016
#define GL_FUNC_REVERSE_SUBTRACT 0x7017
#define GL_FUNC_SUBTRACT 0x7018
#define GL_GEQUAL 0x7019
#define GL_GREATER 0x701A
#define GL_INCR 0x701B
#define GL_INCR_WRAP 0x701C
#define GL_INVERT 0x701D
#define GL_KEEP 0x701E
#define GL_LESS 0x701F
#define GL_MAX_LIGHTS 0x0D31
#define GL_NO_ERROR 0
#define GL_LIGHT0 0x7020
#define GL_LIGHTING_BIT 0x7021
#define GL_LINE 0x7022
#define GL_LINEAR 0x7023
#define GL_LINEAR_ATTENUATION 0x7024
#define GL_LOWER_LEFT 0x7025
#define GL_MAX 0x7026
#define GL_MIN 0x7027
#define GL_NEVER 0x7028
#define GL_NICEST 0x7029
#define GL_NOTEQUAL 0x702A
#define GL_ONE_MINUS_CONSTANT_ALPHA 0x702B
#define GL_ONE_MINUS_CONSTANT_COLOR 0x702C
#define GL_ONE_MINUS_DST_ALPHA 0x702D
#define GL_ONE_MINUS_DST_COLOR 0x702E
#define GL_ONE_MINUS_SRC_ALPHA 0x702F
#define GL_ONE_MINUS_SRC_COLOR 0x7030
#define GL_POINT 0x7031
#define GL_POLYGON_BIT 0x7032
#define GL_POLYGON_MODE 0x7033
#define GL_POSITION 0x7034
#define GL_QUADRATIC_ATTENUATION 0x7035
#define GL_REPLACE 0x7036
#define GL_SPECULAR 0x7037
#define GL_SRC_ALPHA_SATURATE 0x7038
#define GL_SRC_COLOR 0x7039
#define GL_TRUE 0x703A
#define GL_UPPER_LEFT 0x703B
#define GL_ZERO 0x703C
#define GL_AMBIENT 0x703D
#define GL_POLYGON_OFFSET_FILL 0x703E
#define GL_POLYGON_OFFSET_LINE 0x703F
#define GL_POLYGON_OFFSET_POINT 0x7040
#define GL_DEPTH_TEST 0x7041
#define GL_MODELVIEW 0x7042
#define GL_PROJECTION 0x7043
#define GL_TEXTURE_2D 0x7044
#define GL_SMOOTH 0x7045
#define GL_FLAT 0x7046
static inline void glLoadIdentity(void) {}
static inline void glLightfv(GLenum, GLenum, const GLfloat *) {}
static inline void glLightf(GLenum, GLenum, GLfloat) {}
static inline void glTranslatef(GLfloat, GLfloat, GLfloat) {}
static inline void glAlphaFunc(GLenum, GLclampf) {}
static inline void glBlendColor(GLclampf, GLclampf, GLclampf, GLclampf) {}
static inline void glBlendEquation(GLenum) {}
static inline void glColorMask(GLboolean, GLboolean, GLboolean, GLboolean) {}
static inline void glCullFace(GLenum) {}
static inline void glDepthFunc(GLenum) {}
static inline void glDepthMask(GLboolean) {}
static inline void glDepthRange(GLclampd, GLclampd) {}
static inline void glFogf(GLenum, GLfloat) {}
static inline void glFogfv(GLenum, const GLfloat *) {}
static inline void glFogi(GLenum, GLint) {}
static inline void glFrontFace(GLenum) {}
static inline void glHint(GLenum, GLenum) {}
static inline void glPointParameterf(GLenum, GLfloat) {}
static inline void glPointParameterfv(GLenum, const GLfloat *) {}
static inline void glPointParameteri(GLenum, GLint) {}
static inline void glPointSize(GLfloat) {}
static inline void glPolygonMode(GLenum, GLenum) {}
static inline void glPolygonOffset(GLfloat, GLfloat) {}
static inline void glStencilFunc(GLenum, GLint, GLuint) {}
static inline void glStencilOp(GLenum, GLenum, GLenum) {}
static inline void glGetFloatv(GLenum, GLfloat *) {}
static inline void glGetIntegerv(GLenum, GLint *) {}
static inline void glGetBooleanv(GLenum, GLboolean *) {}
static inline GLenum glGetError(void) { return 0; }
static inline void glMaterialfv(GLenum, GLenum, const GLfloat *) {}
static inline void glMatrixMode(GLenum) {}
static inline void glBegin(GLenum) {}
static inline void glEnd(void) {}
static inline void glBlendFunc(GLenum, GLenum) {}
static inline void glCallList(GLuint) {}
static inline void glColor3f(GLfloat, GLfloat, GLfloat) {}
static inline void glColor4f(GLfloat, GLfloat, GLfloat, GLfloat) {}
static inline void glColorMaterial(GLenum, GLenum) {}
static inline void glDeleteLists(GLuint, GLsizei) {}
static inline void glDisable(GLenum) {}
static inline void glEnable(GLenum) {}
static inline void glEnableClientState(GLenum) {}
static inline void glDisableClientState(GLenum) {}
static inline void glDrawElements(GLenum, GLsizei, GLenum, const void *) {}
static inline void glEndList(void) {}
static inline GLuint glGenLists(GLsizei) { return 0; }
static inline void glGetDoublev(GLenum, GLdouble *) {}
static inline void glNewList(GLuint, GLenum) {}
static inline void glNormal3f(GLfloat, GLfloat, GLfloat) {}
static inline void glNormal3d(GLdouble, GLdouble, GLdouble) {}
static inline void glNormal3dv(const GLdouble *) {}
static inline void glNormalPointer(GLenum, GLsizei, const void *) {}
static inline void glPopAttrib(void) {}
static inline void glPushAttrib(GLbitfield) {}
static inline void glPopMatrix(void) {}
static inline void glPushMatrix(void) {}
static inline void glTexCoord2d(GLdouble, GLdouble) {}
static inline void glTexCoord2dv(const GLdouble *) {}
static inline void glTexCoordPointer(GLint, GLenum, GLsizei, const void *) {}
static inline void glVertex3d(GLdouble, GLdouble, GLdouble) {}
static inline void glVertex3f(GLfloat, GLfloat, GLfloat) {}
static inline void glVertex3dv(const GLdouble *) {}
static inline void glVertexPointer(GLint, GLenum, GLsizei, const void *) {}
static inline void glMultMatrixd(const GLdouble *) {}
static inline void glLoadMatrixd(const GLdouble *) {}
static inline void glColor3d(GLdouble, GLdouble, GLdouble) {}
static inline void glColor3dv(const GLdouble *) {}
#endif
