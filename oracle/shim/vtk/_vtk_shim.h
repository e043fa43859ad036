// Stand-in for the handful of VTK classes MRAG's VTK writers name. VTK is not
// installed; the oracle never writes VTK files, so every writer is a no-op.
// Arrays still allocate, because the writers fill them before writing.
#pragma once
#pragma push_macro("min")
#pragma push_macro("max")
#undef min
#undef max
#include <cstdlib>
#include <vector>
#pragma pop_macro("max")
#pragma pop_macro("min")
typedef long long vtkIdType;
#define VTK_PIXEL 8
#define VTK_VOXEL 11
#define VTK_QUAD 9
#define VTK_HEXAHEDRON 12
class vtkShimObject {
public:
    virtual ~vtkShimObject() {}
    void Delete() { delete this; }
};
class vtkFloatArray : public vtkShimObject {
    std::vector<float> d_;
    int nc_ = 1;
public:
    static vtkFloatArray *New() { return new vtkFloatArray; }
    void SetNumberOfComponents(int n) { nc_ = n; }
    void SetName(const char *) {}
    void SetNumberOfTuples(vtkIdType n) { d_.assign((size_t)n * nc_, 0.f); }
    void *GetVoidPointer(vtkIdType i) { return d_.empty() ? nullptr : &d_[(size_t)i]; }
};
class vtkPoints : public vtkShimObject {
    std::vector<float> d_;
public:
    static vtkPoints *New() { return new vtkPoints; }
    void SetNumberOfPoints(vtkIdType n) { d_.assign((size_t)n * 3, 0.f); }
    void *GetVoidPointer(vtkIdType i) { return d_.empty() ? nullptr : &d_[(size_t)i]; }
};
class vtkDataSetAttributes {
public:
    void AddArray(vtkFloatArray *) {}
};
class vtkPointData : public vtkDataSetAttributes {};
class vtkCellData : public vtkDataSetAttributes {};
class vtkCell {};
class vtkUnstructuredGrid : public vtkShimObject {
    vtkPointData pd_;
    vtkCellData cd_;
public:
    static vtkUnstructuredGrid *New() { return new vtkUnstructuredGrid; }
    void SetPoints(vtkPoints *) {}
    void Allocate(vtkIdType) {}
    void InsertNextCell(int, int, vtkIdType *) {}
    vtkPointData *GetPointData() { return &pd_; }
    vtkCellData *GetCellData() { return &cd_; }
};
class vtkXMLUnstructuredGridWriter : public vtkShimObject {
public:
    static vtkXMLUnstructuredGridWriter *New() { return new vtkXMLUnstructuredGridWriter; }
    void SetFileName(const char *) {}
    void SetInput(vtkUnstructuredGrid *) {}
    void Write() {}
};
class vtkUnstructuredGridWriter : public vtkXMLUnstructuredGridWriter {
public:
    static vtkUnstructuredGridWriter *New() { return new vtkUnstructuredGridWriter; }
};
