/******************************************************************************
peaks.cu -- measures the SIMT peaks the solver's roofline is quoted against:
FP32 FMA, FP64 FMA and the FP32 reciprocal (special-function unit)
throughput, each from independent dependency chains in every thread of a
grid of several CTAs per SM, timed with CUDA events.  Prints one JSON line.
Built by ccf_gb300/build.py as ccf_gb300/lib/ccf_peaks.
******************************************************************************/
#include <cuda_runtime.h>

#include <cstdio>

constexpr int CHAINS = 8;

__global__ void ffma_kernel(float* out, int iters, float x, float y)
{
	float a[CHAINS];
	for (int c = 0; c < CHAINS; c++) a[c] = threadIdx.x * 1e-3f + c;
	for (int i = 0; i < iters; i++)
	{
#pragma unroll
		for (int c = 0; c < CHAINS; c++) a[c] = fmaf(a[c], x, y);
	}
	float s = 0;
	for (int c = 0; c < CHAINS; c++) s += a[c];
	if (s == 1234.5f) out[0] = s;
}

__global__ void dfma_kernel(double* out, int iters, double x, double y)
{
	double a[CHAINS];
	for (int c = 0; c < CHAINS; c++) a[c] = threadIdx.x * 1e-3 + c;
	for (int i = 0; i < iters; i++)
	{
#pragma unroll
		for (int c = 0; c < CHAINS; c++) a[c] = fma(a[c], x, y);
	}
	double s = 0;
	for (int c = 0; c < CHAINS; c++) s += a[c];
	if (s == 1234.5) out[0] = s;
}

__global__ void rcp_kernel(float* out, int iters)
{
	float a[CHAINS];
	for (int c = 0; c < CHAINS; c++) a[c] = 1.5f + threadIdx.x * 1e-4f + c;
	for (int i = 0; i < iters; i++)
	{
#pragma unroll
		for (int c = 0; c < CHAINS; c++)
		{
			float r;
			asm volatile("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a[c]));
			a[c] = r;
		}
	}
	float s = 0;
	for (int c = 0; c < CHAINS; c++) s += a[c];
	if (s == 1234.5f) out[0] = s;
}

template <class K>
static double time_ms(K launch)
{
	cudaEvent_t a, b;
	cudaEventCreate(&a);
	cudaEventCreate(&b);
	launch();
	cudaDeviceSynchronize();
	float best = 1e30f;
	for (int r = 0; r < 5; r++)
	{
		cudaEventRecord(a);
		launch();
		cudaEventRecord(b);
		cudaEventSynchronize(b);
		float ms;
		cudaEventElapsedTime(&ms, a, b);
		if (ms < best) best = ms;
	}
	return best;
}

int main()
{
	cudaDeviceProp prop;
	if (cudaGetDeviceProperties(&prop, 0) != cudaSuccess)
	{
		std::printf("{\"error\": \"no device\"}\n");
		return 1;
	}
	const int sms = prop.multiProcessorCount;
	const int threads = 256, blocks = sms * 8;
	float* fo;
	double* dout;
	cudaMalloc(&fo, 64);
	cudaMalloc(&dout, 64);
	const int fi = 1 << 16, di = 1 << 11, ri = 1 << 13;
	double t32 = time_ms([&] { ffma_kernel<<<blocks, threads>>>(fo, fi, 0.999999f, 1e-7f); });
	double t64 = time_ms([&] { dfma_kernel<<<blocks, threads>>>(dout, di, 0.999999999, 1e-9); });
	double tr = time_ms([&] { rcp_kernel<<<blocks, threads>>>(fo, ri); });
	double n = (double)blocks * threads * CHAINS;
	double fp32 = 2.0 * n * fi / (t32 * 1e-3) / 1e12;
	double fp64 = 2.0 * n * di / (t64 * 1e-3) / 1e12;
	double rcp = n * ri / (tr * 1e-3) / 1e12;
	std::printf("{\"fp32_tflops\": %.3f, \"fp64_tflops\": %.4f, \"rcp32_tops\": %.3f, \"sms\": %d}\n",
		fp32, fp64, rcp, sms);
	cudaFree(fo);
	cudaFree(dout);
	return 0;
}
