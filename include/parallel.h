/*
 * parallel.h -- thread controls of UltimateKalman's parallel smoothers
 * (c/parallel.h:31-32), kept so that clients which set them still build and
 * link.  libukgpu.so sizes its GPU launches itself; both calls are accepted
 * and have no effect.
 */
#ifndef PARALLEL_H
#define PARALLEL_H

#ifdef __cplusplus
extern "C" {
#endif

void parallel_set_thread_limit(int number_of_threads);
void parallel_set_blocksize(int blocksize_in);

#ifdef __cplusplus
}
#endif

#endif
