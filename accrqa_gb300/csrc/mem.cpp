// mem.cpp -- the Mem array handle of the reference's C ABI
// (include/AccRQA_utilities_mem.hpp:16-152): a reference-counted
// N-dimensional view of host or device memory.  The Python package wraps
// numpy arrays with mem_create_wrapper and reads them back through the
// accessors; functions keep the reference's null-handle behaviour.
#include <cuda_runtime_api.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "accrqa_gb300.h"

struct Mem {
    MemType type;
    MemLocation location;
    int32_t c_contiguous;
    int32_t owner;          // data allocated here (freed with the handle)
    int32_t read_only;
    int32_t ndim;
    int64_t nelem;
    int32_t refs;
    int64_t *shape;
    int64_t *stride;        // bytes, numpy convention
    void *data;
};

static void mem_msg(const char *m) { std::fprintf(stderr, "AccRQA-GB300 mem: %s\n", m); }

extern "C" {

int64_t mem_type_size(MemType type) {
    switch (type) {
        case MEM_CHAR: return 1;
        case MEM_INT: return (int64_t)sizeof(int);
        case MEM_FLOAT: return 4;
        case MEM_DOUBLE: return 8;
        case MEM_COMPLEX_FLOAT: return 8;
        case MEM_COMPLEX_DOUBLE: return 16;
        default: return 0;
    }
}

MemType mem_type_from_int(int32_t type) {
    switch (type) {
        case MEM_VOID: case MEM_CHAR: case MEM_INT: case MEM_FLOAT: case MEM_DOUBLE:
        case MEM_COMPLEX: case MEM_COMPLEX_FLOAT: case MEM_COMPLEX_DOUBLE:
            return (MemType)type;
        default:
            return MEM_VOID;
    }
}

Mem *mem_create_wrapper(void *data, MemType type, MemLocation location, int32_t num_dims,
                        const int64_t *shape, const int64_t *stride, Accrqa_Error *status) {
    Mem *m = (Mem *)std::calloc(1, sizeof(Mem));
    if (!m) {
        *status = ERR_MEM_ALLOC_FAILURE;
        mem_msg("handle allocation failed");
        return m;
    }
    m->data = data;
    m->refs = 1;
    m->type = type;
    m->location = location;
    m->ndim = num_dims;
    m->nelem = 1;
    const int64_t esize = mem_type_size(type);
    if (esize <= 0) {
        *status = ERR_DATA_TYPE;
        mem_msg("unsupported data type");
        return m;
    }
    if (num_dims <= 0) return m;   // a scalar
    m->shape = (int64_t *)std::calloc((size_t)num_dims, sizeof(int64_t));
    m->stride = (int64_t *)std::calloc((size_t)num_dims, sizeof(int64_t));
    if (!m->shape || !m->stride) {
        *status = ERR_MEM_ALLOC_FAILURE;
        mem_msg("shape allocation failed");
        return m;
    }
    int64_t contiguous = esize;
    m->c_contiguous = 1;
    for (int32_t d = num_dims - 1; d >= 0; d--) {
        m->shape[d] = shape[d];
        m->stride[d] = stride ? stride[d] : m->nelem * esize;
        if (m->stride[d] != contiguous) m->c_contiguous = 0;
        contiguous *= shape[d];
        m->nelem *= shape[d];
    }
    return m;
}

static void mem_allocate(Mem *m, Accrqa_Error *status) {
    m->owner = 1;
    const size_t bytes = (size_t)m->nelem * (size_t)mem_type_size(m->type);
    if (*status || bytes == 0) return;
    if (m->location == MEM_CPU) {
        m->data = std::calloc(bytes, 1);
        if (!m->data) {
            *status = ERR_MEM_ALLOC_FAILURE;
            mem_msg("host allocation failed");
        }
    } else if (m->location == MEM_GPU) {
        cudaError_t e = cudaMalloc(&m->data, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            m->data = nullptr;
            *status = ERR_MEM_ALLOC_FAILURE;
            mem_msg("device allocation failed");
        }
    } else {
        *status = ERR_MEM_LOCATION;
        mem_msg("unsupported memory location");
    }
}

Mem *mem_create(MemType type, MemLocation location, int32_t num_dims, const int64_t *shape,
                const int64_t *stride, Accrqa_Error *status) {
    Mem *m = mem_create_wrapper(nullptr, type, location, num_dims, shape, stride, status);
    if (m) mem_allocate(m, status);
    return m;
}

void mem_copy_contents(Mem *dst, const Mem *src, int64_t offset_dst, int64_t offset_src,
                       int64_t num_elements, Accrqa_Error *status) {
    if (*status || !dst || !src || !dst->data || !src->data) return;
    if (src->nelem == 0 || num_elements == 0) return;
    const int64_t es = mem_type_size(src->type);
    const size_t bytes = (size_t)es * (size_t)num_elements;
    const char *ps = (const char *)src->data + es * offset_src;
    char *pd = (char *)dst->data + es * offset_dst;
    if (src->location == MEM_CPU && dst->location == MEM_CPU) {
        std::memcpy(pd, ps, bytes);
        return;
    }
    cudaMemcpyKind kind;
    if (src->location == MEM_CPU && dst->location == MEM_GPU) kind = cudaMemcpyHostToDevice;
    else if (src->location == MEM_GPU && dst->location == MEM_CPU) kind = cudaMemcpyDeviceToHost;
    else if (src->location == MEM_GPU && dst->location == MEM_GPU) kind = cudaMemcpyDeviceToDevice;
    else {
        *status = ERR_MEM_LOCATION;
        mem_msg("unsupported memory location");
        return;
    }
    if (cudaMemcpy(pd, ps, bytes, kind) != cudaSuccess) {
        cudaGetLastError();
        *status = ERR_MEM_COPY_FAILURE;
        mem_msg("cudaMemcpy failed");
    }
}

Mem *mem_create_copy(const Mem *src, MemLocation location, Accrqa_Error *status) {
    Mem *m = mem_create_wrapper(nullptr, src->type, location, src->ndim, src->shape,
                                src->stride, status);
    if (!m) return m;
    mem_allocate(m, status);
    mem_copy_contents(m, src, 0, 0, src->nelem, status);
    return m;
}

void mem_clear_contents(Mem *mem, Accrqa_Error *status) {
    if (*status || !mem || mem->nelem == 0) return;
    const size_t bytes = (size_t)mem->nelem * (size_t)mem_type_size(mem->type);
    if (mem->location == MEM_CPU) {
        std::memset(mem->data, 0, bytes);
    } else if (mem->location == MEM_GPU) {
        if (cudaMemset(mem->data, 0, bytes) != cudaSuccess) {
            cudaGetLastError();
            *status = ERR_MEM_LOCATION;
        }
    } else {
        *status = ERR_MEM_LOCATION;
    }
}

void *mem_data(Mem *mem) { return mem ? mem->data : nullptr; }
const void *mem_data_const(const Mem *mem) { return mem ? mem->data : nullptr; }

// The reference returns the address of the handle's data pointer here
// (src/AccRQA_utilities_mem.cpp:261-283); kept for ABI compatibility.
void *mem_gpu_buffer(Mem *mem, Accrqa_Error *status) {
    if (*status || !mem) return nullptr;
    if (mem->location != MEM_GPU) {
        *status = ERR_MEM_LOCATION;
        mem_msg("requested buffer is not in GPU memory");
        return nullptr;
    }
    return &mem->data;
}

const void *mem_gpu_buffer_const(const Mem *mem, Accrqa_Error *status) {
    if (*status || !mem) return nullptr;
    if (mem->location != MEM_GPU) {
        *status = ERR_MEM_LOCATION;
        mem_msg("requested buffer is not in GPU memory");
        return nullptr;
    }
    return &mem->data;
}

void mem_free(Mem *mem) {
    if (!mem) return;
    if (--mem->refs > 0) return;
    if (mem->owner && mem->data) {
        if (mem->location == MEM_CPU) std::free(mem->data);
        else if (mem->location == MEM_GPU) cudaFree(mem->data);
    }
    std::free(mem->shape);
    std::free(mem->stride);
    std::free(mem);
}

int32_t mem_is_c_contiguous(const Mem *mem) { return (!mem || !mem->data) ? 0 : mem->c_contiguous; }
int32_t mem_is_complex(const Mem *mem) {
    return (!mem || !mem->data) ? 0 : ((mem->type & MEM_COMPLEX) == MEM_COMPLEX);
}
int32_t mem_is_read_only(const Mem *mem) { return (!mem || !mem->data) ? 1 : mem->read_only; }
MemLocation mem_location(const Mem *mem) { return mem ? mem->location : MEM_CPU; }
int32_t mem_num_dims(const Mem *mem) { return mem ? mem->ndim : 0; }
int64_t mem_num_elements(const Mem *mem) { return (!mem || !mem->data) ? 0 : mem->nelem; }

void mem_random_fill(Mem *mem, Accrqa_Error *status) {
    if (*status || !mem) return;
    if (mem->location != MEM_CPU) {
        *status = ERR_MEM_LOCATION;
        return;
    }
    int64_t n = mem->nelem * (mem_is_complex(mem) ? 2 : 1);
    const int prec = mem->type & 0x0F;
    if (prec == MEM_FLOAT) {
        float *d = (float *)mem->data;
        for (int64_t i = 0; i < n; i++) d[i] = (float)std::rand() / (float)RAND_MAX;
    } else if (prec == MEM_DOUBLE) {
        double *d = (double *)mem->data;
        for (int64_t i = 0; i < n; i++) d[i] = (double)std::rand() / (double)RAND_MAX;
    }
}

void mem_ref_dec(Mem *mem) { mem_free(mem); }
Mem *mem_ref_inc(Mem *mem) {
    if (!mem) return nullptr;
    mem->refs++;
    return mem;
}
void mem_set_read_only(Mem *mem, int32_t value) {
    if (mem) mem->read_only = value;
}
int64_t mem_shape_dim(const Mem *mem, int32_t dim) {
    return (!mem || dim < 0 || dim >= mem->ndim) ? 0 : mem->shape[dim];
}
int64_t mem_stride_dim(const Mem *mem, int32_t dim) {
    return (!mem || dim < 0 || dim >= mem->ndim) ? 0 : mem->stride[dim];
}
MemType mem_type(const Mem *mem) { return mem ? mem->type : MEM_VOID; }

int32_t mem_assert(Mem *mem, MemType type, MemLocation location) {
    return (mem && mem->type == type && mem->location == location) ? 0 : 1;
}

int32_t mem_assert_type(Mem *A, Mem *B, Accrqa_Error *status) {
    if (!A || !B) {
        *status = ERR_MEM_ALLOC_FAILURE;
        return 1;
    }
    if (mem_type(A) != mem_type(B)) {
        *status = ERR_DATA_TYPE;
        return 1;
    }
    return 0;
}

int32_t mem_assert_location(Mem *A, Mem *B, Accrqa_Error *status) {
    if (!A || !B) {
        *status = ERR_MEM_ALLOC_FAILURE;
        return 1;
    }
    if (mem_location(A) != mem_location(B)) {
        *status = ERR_MEM_LOCATION;
        return 1;
    }
    return 0;
}

int32_t mem_assert_nElements(Mem *A, Mem *B, Accrqa_Error *status) {
    if (!A || !B) {
        *status = ERR_MEM_ALLOC_FAILURE;
        return 1;
    }
    if (mem_num_elements(A) != mem_num_elements(B)) {
        *status = ERR_INVALID_ARGUMENT;
        return 1;
    }
    return 0;
}

int32_t mem_assert_null(Mem *A, Accrqa_Error *status) {
    if (!A) {
        *status = ERR_MEM_ALLOC_FAILURE;
        return 1;
    }
    return 0;
}

}  // extern "C"
