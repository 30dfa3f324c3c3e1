// Output frames on the device: the payload of write_frame_bin
// (solver_output.cu:259-316) built from the engine's state, so that only the
// finished frame crosses to the host.
//
// Frame layout (the file's bytes): int32 count of active particles, then their
// positions (float32 x, y, z each times the length factor), then their radii
// (float32 times the length factor), in pId order.  A particle counts as
// active when its status is 1 (a particle leaving the box this step has
// status 2: the reference deactivates it before writing, main.cu:312-321).
//
// Compiled with -fmad=false: (float)(x * lf) is the reference's conversion.
#include "gdem_internal.cuh"

namespace gdem {

namespace {

constexpr int kScanBlock = 1024;

// pId-order copy of what the frame needs
template <class T>
__global__ void k_frame_gather(View<T> v, float* __restrict__ posf, float* __restrict__ rf, int* __restrict__ flag,
                               double lf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.n) return;
    const Ctl* ctl = v.ctl;
    const SBank<T> S = v.S[ctl->s];
    const int q = v.P[ctl->p].pid[i];
    const double4_32a p = load_pos(S, i);
    flag[q] = S.rot[i].w == 1 ? 1 : 0;
    posf[3 * q] = (float)(p.x * lf);
    posf[3 * q + 1] = (float)(p.y * lf);
    posf[3 * q + 2] = (float)(p.z * lf);
    rf[q] = (float)(p.w * lf);
}

// exclusive scan of the flags inside each block of kScanBlock, and the block sums
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(const int* __restrict__ flag, int* __restrict__ offs,
                                                            int* __restrict__ bsum, int n) {
    __shared__ int ws[32];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int x = i < n ? flag[i] : 0;
    int incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) ws[w] = incl;
    __syncthreads();
    if (w == 0) {
        int s = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        ws[lane] = s;
    }
    __syncthreads();
    const int before = (w ? ws[w - 1] : 0) + incl - x;
    if (i < n) offs[i] = before;
    if (threadIdx.x == kScanBlock - 1) bsum[blockIdx.x] = before + x;
}

// exclusive scan of the block sums (one block) and the total
__global__ void __launch_bounds__(kScanBlock) k_scan_sums(int* __restrict__ bsum, int nb, int* __restrict__ total) {
    __shared__ int ws[32];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += kScanBlock) {
        const int i = base + threadIdx.x;
        const int x = i < nb ? bsum[i] : 0;
        int incl = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) ws[w] = incl;
        __syncthreads();
        if (w == 0) {
            int s = ws[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            ws[lane] = s;
        }
        __syncthreads();
        const int c = carry;
        if (i < nb) bsum[i] = c + (w ? ws[w - 1] : 0) + incl - x;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry = c + ws[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// the frame: count, positions, radii of the active particles in pId order
__global__ void k_frame_scatter(const float* __restrict__ posf, const float* __restrict__ rf,
                                const int* __restrict__ flag, const int* __restrict__ offs,
                                const int* __restrict__ bsum, const int* __restrict__ total, char* __restrict__ frame,
                                int n) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int count = *total;
    if (q == 0) *reinterpret_cast<int*>(frame) = count;
    if (q >= n || !flag[q]) return;
    const int k = bsum[q / kScanBlock] + offs[q];
    float* pos = reinterpret_cast<float*>(frame + 4);
    float* rad = reinterpret_cast<float*>(frame + 4 + 12 * (size_t)count);
    pos[3 * (size_t)k] = posf[3 * q];
    pos[3 * (size_t)k + 1] = posf[3 * q + 1];
    pos[3 * (size_t)k + 2] = posf[3 * q + 2];
    rad[k] = rf[q];
}

}  // namespace

size_t frame_scratch_bytes(int n) {
    const int nb = (n + kScanBlock - 1) / kScanBlock;
    return sizeof(float) * 4 * (size_t)n + sizeof(int) * (2 * (size_t)n + nb + 1) + 4 * 256;
}

size_t frame_bytes(int n) { return 4 + 16 * (size_t)n; }

template <class T>
void launch_frame(const View<T>& v, void* scratch, char* frame, double lf, cudaStream_t st) {
    const int n = v.n;
    const int nb = (n + kScanBlock - 1) / kScanBlock;
    char* s = static_cast<char*>(scratch);
    float* posf = reinterpret_cast<float*>(s);
    float* rf = posf + 3 * (size_t)n;
    int* flag = reinterpret_cast<int*>(rf + n);
    int* offs = flag + n;
    int* bsum = offs + n;
    int* total = bsum + nb;
    const int g = (n + kBlock - 1) / kBlock;
    k_frame_gather<T><<<g, kBlock, 0, st>>>(v, posf, rf, flag, lf);
    k_scan_blocks<<<nb, kScanBlock, 0, st>>>(flag, offs, bsum, n);
    k_scan_sums<<<1, kScanBlock, 0, st>>>(bsum, nb, total);
    k_frame_scatter<<<g, kBlock, 0, st>>>(posf, rf, flag, offs, bsum, total, frame, n);
}

template void launch_frame<FP64>(const View<FP64>&, void*, char*, double, cudaStream_t);
template void launch_frame<Mixed>(const View<Mixed>&, void*, char*, double, cudaStream_t);

}  // namespace gdem
