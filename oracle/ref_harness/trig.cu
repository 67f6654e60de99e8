// The device's single-precision cos and sin of n angles (radians): the
// values the reference's GPU TTI programs compute for their tilt inside
// their kernels (cos(theta[id]), sin(theta[id]) of a float,
// 2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:106-107).  Test
// infrastructure: the CPU oracle cannot reproduce the device's cosf/sinf
// bit for bit, so the tests hand it these values (oracle/refgpu.py,
// cuda_trig).  Built with contraction off, as the library is.
extern "C" __global__ void k_ref_trig(const float *th, float *c, float *s, long n) {
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        c[k] = cosf(th[k]);
        s[k] = sinf(th[k]);
    }
}
