/*
 * Linux stand-in for DXViewer's Win32App.h, the un-vendored submodule header
 * that the reference's src/Kobayashi.h:2 includes.  TEST INFRASTRUCTURE ONLY:
 * it lets the reference's own src/Kobayashi.cpp compile unmodified into the
 * oracle/_ref libraries.  Everything here is a do-nothing declaration of the
 * Win32 / Direct3D / DXViewer names that Kobayashi.cpp mentions; the only
 * definition that reaches the numerics is PI_F, which DXViewer defines and
 * which is not vendored: it is written as the double literal of pi so that the
 * FP64 build (float -> double) sees RN(pi) and the FP32 build sees RN32(pi).
 * The ISimulation method list mirrors the overrides in src/Kobayashi.h:41-66.
 */
#pragma once
#include <vector>
#include <string>
#include <cmath>
#include <cfloat>
#include <ctime>

#define TRUE 1
typedef unsigned int UINT;
typedef void* HWND;
typedef void* HINSTANCE;
typedef void* HMENU;
typedef unsigned long WPARAM;
typedef long LPARAM;
#define LOWORD(w) ((int)((w) & 0xffff))
#define HIWORD(w) ((int)(((w) >> 16) & 0xffff))
enum {
    WS_CHILD = 1, WS_VISIBLE = 2, BS_PUSHBUTTON = 4, SBS_HORZ = 8, SB_CTL = 2,
    SB_LINELEFT = 0, SB_LINERIGHT = 1, SB_PAGELEFT = 2, SB_PAGERIGHT = 3, SB_THUMBTRACK = 5,
    D3D11_PRIMITIVE_TOPOLOGY_TRIANGLELIST = 4
};
inline HWND CreateWindow(const wchar_t*, const wchar_t*, int, int, int, int, int, HWND, HMENU, HINSTANCE, void*) { return nullptr; }
inline void SetScrollRange(HWND, int, int, int, int) {}
inline void SetScrollPos(HWND, int, int, int) {}
inline void SetDlgItemText(HWND, int, const wchar_t*) {}
inline HWND GetDlgItem(HWND, int) { return nullptr; }
inline void EnableWindow(HWND, bool) {}
inline void SetTimer(HWND, int, int, void*) {}
inline void KillTimer(HWND, int) {}

static const float PI_F = 3.14159265358979323846;

namespace DirectX {
struct XMFLOAT2 { float x, y; XMFLOAT2(float a, float b) : x(a), y(b) {} };
struct XMFLOAT3 { float x, y, z; XMFLOAT3() = default; XMFLOAT3(float a, float b, float c) : x(a), y(b), z(c) {} };
struct XMFLOAT4 { float x, y, z, w; XMFLOAT4() = default; XMFLOAT4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {} };
struct XMINT2 { int x, y; };
struct XMINT3 { int x, y, z; };
struct XMFLOAT4X4 { float m[16]; };
}
namespace DXViewer {
namespace xmfloat3 {
inline DirectX::XMFLOAT3 operator*(DirectX::XMFLOAT3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline DirectX::XMFLOAT3 operator+(DirectX::XMFLOAT3 a, DirectX::XMFLOAT3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
}
namespace util {
inline DirectX::XMFLOAT4X4 transformMatrix(float, float, float, float = 1.0f) { return {}; }
}
}
namespace Microsoft { namespace WRL {
template <class T> struct ComPtr { T* operator->() { return p; } T* p = nullptr; };
} }
struct ID3D12GraphicsCommandList {
    void IASetPrimitiveTopology(int) {}
    void DrawIndexedInstanced(int, int, int, int, int) {}
};
struct Vertex { DirectX::XMFLOAT3 pos; Vertex(DirectX::XMFLOAT3 p) : pos(p) {} };
struct ConstantBuffer { DirectX::XMFLOAT4X4 world, worldViewProj, transInvWorld; DirectX::XMFLOAT4 color; };
struct DX12App { void update() {} void draw() {} void resetSimulationState() {} };

struct ISimulation {
    virtual ~ISimulation() {}
    virtual void iUpdate() = 0;
    virtual void iResetSimulationState(std::vector<ConstantBuffer>&) = 0;
    virtual std::vector<Vertex>& iGetVertices() = 0;
    virtual std::vector<unsigned int>& iGetIndices() = 0;
    virtual UINT iGetVertexBufferSize() = 0;
    virtual UINT iGetIndexBufferSize() = 0;
    virtual void iCreateObject(std::vector<ConstantBuffer>&) = 0;
    virtual void iUpdateConstantBuffer(std::vector<ConstantBuffer>&, int) = 0;
    virtual void iDraw(Microsoft::WRL::ComPtr<ID3D12GraphicsCommandList>&, int, UINT, int) = 0;
    virtual void iSetDXApp(DX12App*) = 0;
    virtual UINT iGetConstantBufferSize() = 0;
    virtual DirectX::XMINT3 iGetObjectCount() = 0;
    virtual DirectX::XMFLOAT3 iGetObjectSize() = 0;
    virtual DirectX::XMFLOAT3 iGetObjectPositionOffset() = 0;
    virtual bool iIsUpdated() = 0;
    virtual void iWMCreate(HWND, HINSTANCE) = 0;
    virtual void iWMCommand(HWND, UINT, WPARAM, LPARAM, HINSTANCE) = 0;
    virtual void iWMHScroll(HWND, WPARAM, LPARAM, HINSTANCE) = 0;
    virtual void iWMTimer(HWND) = 0;
    virtual void iWMDestory(HWND) = 0;
};
using std::to_wstring;
