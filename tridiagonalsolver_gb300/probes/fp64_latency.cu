// Dependent-chain latency of DFMA, DMUL, MUFU rcp.f64 and FFMA for 1, 4 and 8
// warps in one CTA (cycles per operation from clock64()).
#include <cstdio>
__device__ unsigned long long g_c[8];
template<int OP> __global__ void k(double* o, double s) {
  double x = s + threadIdx.x*1e-9; float xf = (float)x;
  long long t0 = clock64();
  #pragma unroll 1
  for (int i=0;i<4096;++i){
    #pragma unroll
    for(int u=0;u<8;++u){
      if (OP==0) x = fma(x, 1.0000001, 1e-9);
      if (OP==1) { double r; asm volatile("rcp.approx.ftz.f64 %0,%1;":"=d"(r):"d"(x)); x = r; }
      if (OP==2) xf = fmaf(xf, 1.0000001f, 1e-9f);
      if (OP==3) { float r; asm volatile("rcp.approx.ftz.f32 %0,%1;":"=f"(r):"f"(xf)); xf = r; }
      if (OP==4) x = x * 1.0000001;
    }
  }
  long long t1 = clock64();
  if (threadIdx.x==0 && blockIdx.x==0) g_c[OP] = t1-t0;
  if (x == 1234.5 || xf == 1234.5f) o[0]=x+xf;
}
int main(){ double* o; cudaMalloc(&o,64); unsigned long long c[8];
 const char* nm[5]={"DFMA","rcp.f64","FFMA","rcp.f32","DMUL"};
 for (int w : {1, 4, 8}) {
  k<0><<<1,32*w>>>(o,1.0); k<1><<<1,32*w>>>(o,1.0); k<2><<<1,32*w>>>(o,1.0); k<3><<<1,32*w>>>(o,1.0); k<4><<<1,32*w>>>(o,1.0);
  cudaDeviceSynchronize(); cudaMemcpyFromSymbol(c,g_c,sizeof(c));
  for(int i=0;i<5;++i) printf("warps=%d %-8s %.1f cycles/op (dependent chain)\n", w, nm[i], c[i]/(4096.0*8));
 }
 return 0;}
