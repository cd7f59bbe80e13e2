/*
 * Sequential launch emulation for the reference kernels (test infrastructure only).
 *
 * `kernel<<<grid, block>>>(args)` is rewritten by oracle/build_ref.py into
 * `PCT_LAUNCH(kernel, grid, block)(args)`.  The launcher evaluates the
 * arguments once and then calls the kernel body for every (block, thread) of
 * the grid, x fastest, blocks outermost.  Atomics therefore accumulate in that
 * fixed thread order, which makes every float sum of the reference deterministic.
 */
#ifndef PCT_REF_LAUNCH_H
#define PCT_REF_LAUNCH_H

template <class F> struct PctLauncher {
    dim3 grid, block;
    F body;
    template <class... A> void operator()(A... args) {
        gridDim = grid;
        blockDim = block;
        for (unsigned bz = 0; bz < grid.z; ++bz)
            for (unsigned by = 0; by < grid.y; ++by)
                for (unsigned bx = 0; bx < grid.x; ++bx) {
                    blockIdx.x = bx; blockIdx.y = by; blockIdx.z = bz;
                    for (unsigned tz = 0; tz < block.z; ++tz)
                        for (unsigned ty = 0; ty < block.y; ++ty)
                            for (unsigned tx = 0; tx < block.x; ++tx) {
                                threadIdx.x = tx; threadIdx.y = ty; threadIdx.z = tz;
                                body(args...);
                            }
                }
    }
};
template <class F> PctLauncher<F> pct_grid(dim3 g, dim3 b, F f) { return PctLauncher<F>{g, b, f}; }
#define PCT_LAUNCH(kernel, g, b) pct_grid(dim3(g), dim3(b), [&](auto... pct_a) { kernel(pct_a...); })

/* Two-phase launch for MSC_edge_detection_GPU: every thread reads the
 * original image and writes only its own voxel
 * (column + row*COLUMNS + slice*COLUMNS*ROWS, .cu:3572), so each thread runs
 * against the original values and its result is parked until the grid ends. */
struct PctTwoPhaseLauncher {
    dim3 grid, block;
    template <class F, class T> void run(F body, T* image) {
        gridDim = grid;
        blockDim = block;
        size_t n = (size_t)grid.x * grid.y * block.x;
        T* out = new T[n];
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx)
                for (unsigned tx = 0; tx < block.x; ++tx) {
                    blockIdx.x = bx; blockIdx.y = by; blockIdx.z = 0;
                    threadIdx.x = tx; threadIdx.y = 0; threadIdx.z = 0;
                    size_t v = bx + (size_t)by * grid.x + (size_t)tx * grid.x * grid.y;
                    T saved = image[v];
                    body(image);
                    out[v] = image[v];
                    image[v] = saved;
                }
        for (size_t v = 0; v < n; ++v) image[v] = out[v];
        delete[] out;
    }
};
template <class F> struct PctTwoPhaseCall {
    PctTwoPhaseLauncher l;
    F body;
    template <class T> void operator()(T* image) { l.run(body, image); }
};
template <class F> PctTwoPhaseCall<F> pct_two_phase(dim3 g, dim3 b, F f) { return PctTwoPhaseCall<F>{{g, b}, f}; }
#define PCT_LAUNCH_TWO_PHASE(kernel, g, b) pct_two_phase(dim3(g), dim3(b), [&](auto... pct_a) { kernel(pct_a...); })

[[noreturn]] void pct_reference_exit(int code);

#endif
