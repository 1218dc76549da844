/*
 * gg_compat.h - the older C entry points that the reference's Python ctypes
 * class binds (src/Python/MultiGPUGridder_Python.py:11-48), exported by
 * libgg_gridder.so so that a script written against them runs unchanged.
 *
 * In the reference these names belong to an extern "C" block that is
 * commented out (src/Gridders/MultiGPUGridder.cpp:492-512), so no library in
 * its tree exports them.  They keep that API's shape: the caller registers
 * host arrays by pointer, the calls have no status (a failure leaves the
 * outputs untouched and its message in gg_global_error()), and the data are
 * in CAS space: SetVolume takes a CAS volume of edge V, Forward_Project writes
 * CAS images of edge SetImgSize()[0], Back_Project back-projects the
 * registered CAS images into a zeroed CAS volume and writes it over the
 * registered volume array (as the reference's GetVolume returns the
 * registered pointer, AbstractGridder.h:95).  The projection kernels are the
 * ones behind gg_forward_project_kernel / gg_back_project_kernel, with the
 * default KB table (getKernelFiltTable(2, 501)) and the mask radius truncated
 * to int as RunKernel does.
 */
#ifndef GG_COMPAT_H
#define GG_COMPAT_H

#ifdef __cplusplus
extern "C" {
#endif

void *Gridder_new(void);
/* Not in the reference's list (it has no delete): frees a Gridder_new object. */
void Gridder_delete(void *gridder);
void *SetNumberGPUs(void *gridder, int numGPUs);   /* one GPU per object; kept for the caller */
void *SetNumberStreams(void *gridder, int nStreams);
void *SetVolume(void *gridder, float *casVolume, int *volSize);   /* volSize = {V, V, V} */
float *GetVolume(void *gridder);                                   /* the registered volume array */
void *ResetVolume(void *gridder);                                  /* zeroes the registered volume array */
void *SetImages(void *gridder, float *casImages);                  /* CAS images for Back_Project */
float *GetImages(void *gridder);      /* images of the last Forward_Project (library-owned unless SetImages) */
void *SetAxes(void *gridder, float *coordAxes, int *axesSize);    /* axesSize[0] = 9 * number of directions */
void *SetImgSize(void *gridder, int *imgSize);                     /* imgSize[0] = CAS image edge */
void *SetMaskRadius(void *gridder, float *maskRadius);
void *Forward_Project(void *gridder);
void *Back_Project(void *gridder);

#ifdef __cplusplus
}
#endif
#endif /* GG_COMPAT_H */
