// icd_min.cpp -- a minimal OpenCL ICD dispatcher for running the reference
// program (mersenne2_gpu.cpp) where the vendor's OpenCL driver is installed
// but no ICD loader (libOpenCL.so.1) is.  Test infrastructure: it serves only
// the timing of the reference's own GPU path (oracle/build_ref.py).
//
// OpenCL's installable-client-driver interface: a vendor library exports
// clGetExtensionFunctionAddress, through which clIcdGetPlatformIDsKHR is found;
// every object the driver hands out (platform, device, context, queue, memory
// object, program, kernel) starts with a pointer to the driver's dispatch
// table, an array of entry points in the order the ICD interface fixes.  The
// entry points below forward each call through the table of the object it
// names.  Before the table serves any other call, two of its slots are checked
// through calls whose answers are known: slot 65 (clGetExtensionFunctionAddress)
// must resolve clIcdGetPlatformIDsKHR to the same function the vendor
// library's exported clGetExtensionFunctionAddress gave, and slot 1
// (clGetPlatformInfo) must report a platform name that contains "NVIDIA";
// otherwise the platform is refused (CL_PLATFORM_NOT_FOUND_KHR).
//
// The vendor library is $M2_OCL_VENDOR_LIB, else libnvidia-opencl.so.1 from
// the dynamic linker's search path.
#include <CL/cl.h>

#include <dlfcn.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace {

// slots of the ICD dispatch table used here
enum Slot {
    kGetPlatformInfo = 1,
    kGetDeviceIDs = 2,
    kGetDeviceInfo = 3,
    kCreateContext = 4,
    kReleaseContext = 7,
    kCreateCommandQueue = 9,
    kReleaseCommandQueue = 11,
    kCreateBuffer = 14,
    kReleaseMemObject = 18,
    kCreateProgramWithSource = 26,
    kReleaseProgram = 29,
    kBuildProgram = 30,
    kGetProgramBuildInfo = 33,
    kCreateKernel = 34,
    kReleaseKernel = 37,
    kSetKernelArg = 38,
    kFinish = 47,
    kEnqueueReadBuffer = 48,
    kEnqueueNDRangeKernel = 59,
    kGetExtensionFunctionAddress = 65,
};

typedef void* Fn;
// the dispatch table of a driver object
inline Fn* table_of(const void* obj) { return *reinterpret_cast<Fn* const*>(obj); }
template <class F> inline F slot(const void* obj, Slot s) { return reinterpret_cast<F>(table_of(obj)[s]); }

typedef cl_int (*IcdGetPlatformIDs)(cl_uint, cl_platform_id*, cl_uint*);
typedef void* (*GetExtAddr)(const char*);

bool g_checked = false, g_ok = false;

bool load_platforms(cl_uint cap, cl_platform_id* out, cl_uint* count) {
    const char* path = std::getenv("M2_OCL_VENDOR_LIB");
    void* lib = dlopen(path && *path ? path : "libnvidia-opencl.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!lib) { std::fprintf(stderr, "icd_min: no vendor OpenCL library (%s)\n", dlerror()); return false; }
    auto ext = reinterpret_cast<GetExtAddr>(dlsym(lib, "clGetExtensionFunctionAddress"));
    if (!ext) { std::fprintf(stderr, "icd_min: the vendor library lacks the ICD entry points\n"); return false; }
    auto get = reinterpret_cast<IcdGetPlatformIDs>(ext("clIcdGetPlatformIDsKHR"));
    if (!get) { std::fprintf(stderr, "icd_min: clIcdGetPlatformIDsKHR not found\n"); return false; }
    cl_uint n = 0;
    if (get(0, nullptr, &n) != CL_SUCCESS || n == 0) return false;
    cl_platform_id ps[16];
    if (n > 16) n = 16;
    if (get(n, ps, nullptr) != CL_SUCCESS) return false;
    typedef cl_int (*PlatformInfo)(cl_platform_id, cl_platform_info, size_t, void*, size_t*);
    for (cl_uint i = 0; i < n; ++i) {
        const void* via_table = slot<GetExtAddr>(ps[i], kGetExtensionFunctionAddress)("clIcdGetPlatformIDsKHR");
        char name[256] = {0};
        const cl_int rc = slot<PlatformInfo>(ps[i], kGetPlatformInfo)(ps[i], CL_PLATFORM_NAME, sizeof(name) - 1, name, nullptr);
        if (via_table != reinterpret_cast<const void*>(get) || rc != CL_SUCCESS || !std::strstr(name, "NVIDIA")) {
            std::fprintf(stderr, "icd_min: platform %u: dispatch-table check failed (slot 65 %s, slot 1 rc %d name '%s'); refused\n",
                         i, via_table == reinterpret_cast<const void*>(get) ? "ok" : "differs", (int)rc, name);
            return false;
        }
        std::fprintf(stderr, "icd_min: platform %u '%s' (dispatch table checked)\n", i, name);
    }
    if (count) *count = n;
    for (cl_uint i = 0; i < n && i < cap; ++i) out[i] = ps[i];
    return true;
}

}  // namespace

extern "C" {

cl_int clGetPlatformIDs(cl_uint num_entries, cl_platform_id* platforms, cl_uint* num_platforms) {
    static cl_platform_id cache[16];
    static cl_uint ncache = 0;
    if (!g_checked) {
        g_checked = true;
        g_ok = load_platforms(16, cache, &ncache);
    }
    if (!g_ok) return CL_PLATFORM_NOT_FOUND_KHR;
    if (num_platforms) *num_platforms = ncache;
    if (platforms) {
        if (num_entries == 0) return CL_INVALID_VALUE;
        for (cl_uint i = 0; i < num_entries && i < ncache; ++i) platforms[i] = cache[i];
    }
    return CL_SUCCESS;
}

cl_int clGetDeviceIDs(cl_platform_id p, cl_device_type t, cl_uint n, cl_device_id* d, cl_uint* nd) {
    return slot<cl_int (*)(cl_platform_id, cl_device_type, cl_uint, cl_device_id*, cl_uint*)>(p, kGetDeviceIDs)(p, t, n, d, nd);
}
cl_int clGetDeviceInfo(cl_device_id d, cl_device_info w, size_t sz, void* v, size_t* ret) {
    return slot<cl_int (*)(cl_device_id, cl_device_info, size_t, void*, size_t*)>(d, kGetDeviceInfo)(d, w, sz, v, ret);
}
cl_context clCreateContext(const cl_context_properties* props, cl_uint nd, const cl_device_id* devs,
                           void (*cb)(const char*, const void*, size_t, void*), void* ud, cl_int* err) {
    if (nd == 0 || !devs) { if (err) *err = CL_INVALID_VALUE; return nullptr; }
    typedef cl_context (*F)(const cl_context_properties*, cl_uint, const cl_device_id*,
                            void (*)(const char*, const void*, size_t, void*), void*, cl_int*);
    return slot<F>(devs[0], kCreateContext)(props, nd, devs, cb, ud, err);
}
cl_command_queue clCreateCommandQueue(cl_context c, cl_device_id d, cl_command_queue_properties pr, cl_int* err) {
    typedef cl_command_queue (*F)(cl_context, cl_device_id, cl_command_queue_properties, cl_int*);
    return slot<F>(c, kCreateCommandQueue)(c, d, pr, err);
}
// the program passes no properties: the same as an OpenCL 1.x in-order queue
cl_command_queue clCreateCommandQueueWithProperties(cl_context c, cl_device_id d, const cl_queue_properties* pr,
                                                    cl_int* err) {
    if (pr && pr[0] != 0) { if (err) *err = CL_INVALID_VALUE; return nullptr; }
    return clCreateCommandQueue(c, d, 0, err);
}
cl_program clCreateProgramWithSource(cl_context c, cl_uint n, const char** s, const size_t* l, cl_int* err) {
    typedef cl_program (*F)(cl_context, cl_uint, const char**, const size_t*, cl_int*);
    return slot<F>(c, kCreateProgramWithSource)(c, n, s, l, err);
}
cl_int clBuildProgram(cl_program p, cl_uint nd, const cl_device_id* d, const char* o, void (*cb)(cl_program, void*),
                      void* ud) {
    typedef cl_int (*F)(cl_program, cl_uint, const cl_device_id*, const char*, void (*)(cl_program, void*), void*);
    return slot<F>(p, kBuildProgram)(p, nd, d, o, cb, ud);
}
cl_int clGetProgramBuildInfo(cl_program p, cl_device_id d, cl_program_build_info w, size_t sz, void* v, size_t* ret) {
    typedef cl_int (*F)(cl_program, cl_device_id, cl_program_build_info, size_t, void*, size_t*);
    return slot<F>(p, kGetProgramBuildInfo)(p, d, w, sz, v, ret);
}
cl_kernel clCreateKernel(cl_program p, const char* name, cl_int* err) {
    return slot<cl_kernel (*)(cl_program, const char*, cl_int*)>(p, kCreateKernel)(p, name, err);
}
cl_int clSetKernelArg(cl_kernel k, cl_uint i, size_t sz, const void* v) {
    return slot<cl_int (*)(cl_kernel, cl_uint, size_t, const void*)>(k, kSetKernelArg)(k, i, sz, v);
}
cl_mem clCreateBuffer(cl_context c, cl_mem_flags f, size_t sz, void* host, cl_int* err) {
    return slot<cl_mem (*)(cl_context, cl_mem_flags, size_t, void*, cl_int*)>(c, kCreateBuffer)(c, f, sz, host, err);
}
cl_int clEnqueueNDRangeKernel(cl_command_queue q, cl_kernel k, cl_uint dim, const size_t* off, const size_t* gs,
                              const size_t* ls, cl_uint ne, const cl_event* ev, cl_event* out) {
    typedef cl_int (*F)(cl_command_queue, cl_kernel, cl_uint, const size_t*, const size_t*, const size_t*, cl_uint,
                        const cl_event*, cl_event*);
    return slot<F>(q, kEnqueueNDRangeKernel)(q, k, dim, off, gs, ls, ne, ev, out);
}
cl_int clEnqueueReadBuffer(cl_command_queue q, cl_mem m, cl_bool blk, size_t off, size_t sz, void* p, cl_uint ne,
                           const cl_event* ev, cl_event* out) {
    typedef cl_int (*F)(cl_command_queue, cl_mem, cl_bool, size_t, size_t, void*, cl_uint, const cl_event*, cl_event*);
    return slot<F>(q, kEnqueueReadBuffer)(q, m, blk, off, sz, p, ne, ev, out);
}
cl_int clFinish(cl_command_queue q) { return slot<cl_int (*)(cl_command_queue)>(q, kFinish)(q); }
cl_int clReleaseKernel(cl_kernel k) { return slot<cl_int (*)(cl_kernel)>(k, kReleaseKernel)(k); }
cl_int clReleaseMemObject(cl_mem m) { return slot<cl_int (*)(cl_mem)>(m, kReleaseMemObject)(m); }
cl_int clReleaseProgram(cl_program p) { return slot<cl_int (*)(cl_program)>(p, kReleaseProgram)(p); }
cl_int clReleaseCommandQueue(cl_command_queue q) { return slot<cl_int (*)(cl_command_queue)>(q, kReleaseCommandQueue)(q); }
cl_int clReleaseContext(cl_context c) { return slot<cl_int (*)(cl_context)>(c, kReleaseContext)(c); }

}  // extern "C"
