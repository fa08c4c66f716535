/* Empty stand-in for <GL/gl.h>, used only when compiling the reference's CUDA kernels into device
 * code (oracle/ref_gpu.py): cuda_gl_interop.h includes it, and the reference's vendored glad.h
 * already defines the GL types it needs.  No graphics API is used or loaded. */
