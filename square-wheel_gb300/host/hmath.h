// Host-side vector/matrix math for the renderer's per-frame setup (camera matrices, plane transforms).
//
// Follows the cgmath 0.18 conventions the reference uses (column-major Matrix4, matrix*vector as a
// linear combination of columns, Quaternion -> Matrix4) and src/common/matrix.rs for the camera.
// cgmath's Matrix4::invert is restated as a cofactor inverse; its exact rounding is not pinned by any
// reference test, and both the GPU path and the oracle consume the matrices computed here.
// Compiled with -ffp-contract=off (host) and --fmad=false (device): every a*b+c is two roundings, as in
// the reference. The vector and matrix operations are __host__ __device__ under nvcc, so the GPU-side
// surface and draw preparation evaluates exactly the same expressions as the host.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define SWH_HD __host__ __device__
#else
#define SWH_HD
#endif

namespace swhost
{

struct Vec2
{
	float x, y;
};
struct Vec3
{
	float x, y, z;
};
struct Vec4
{
	float x, y, z, w;
};

SWH_HD inline Vec2 v2(float x, float y) { return Vec2{x, y}; }
SWH_HD inline Vec3 v3(float x, float y, float z) { return Vec3{x, y, z}; }
SWH_HD inline Vec4 v4(float x, float y, float z, float w) { return Vec4{x, y, z, w}; }
SWH_HD inline Vec3 operator+(Vec3 a, Vec3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
SWH_HD inline Vec3 operator-(Vec3 a, Vec3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
SWH_HD inline Vec3 operator-(Vec3 a) { return v3(-a.x, -a.y, -a.z); }
SWH_HD inline Vec3 operator*(Vec3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
SWH_HD inline Vec3 operator*(float s, Vec3 a) { return v3(s * a.x, s * a.y, s * a.z); }
SWH_HD inline Vec3 operator/(Vec3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
SWH_HD inline Vec2 operator+(Vec2 a, Vec2 b) { return v2(a.x + b.x, a.y + b.y); }
SWH_HD inline Vec2 operator-(Vec2 a, Vec2 b) { return v2(a.x - b.x, a.y - b.y); }
SWH_HD inline Vec2 operator*(Vec2 a, float s) { return v2(a.x * s, a.y * s); }
SWH_HD inline Vec2 operator/(Vec2 a, float s) { return v2(a.x / s, a.y / s); }
// cgmath InnerSpace::dot = (a*b).sum() = ((x*x' + y*y') + z*z') (+ w*w')
SWH_HD inline float dot(Vec2 a, Vec2 b) { return a.x * b.x + a.y * b.y; }
SWH_HD inline float dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SWH_HD inline float dot(Vec4 a, Vec4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
SWH_HD inline float magnitude2(Vec3 a) { return dot(a, a); }
SWH_HD inline float magnitude(Vec3 a) { return sqrtf(magnitude2(a)); }
SWH_HD inline Vec3 cross(Vec3 a, Vec3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
SWH_HD inline Vec4 extend(Vec3 a, float w) { return v4(a.x, a.y, a.z, w); }
SWH_HD inline Vec3 truncate(Vec4 a) { return v3(a.x, a.y, a.z); }
SWH_HD inline Vec4 operator+(Vec4 a, Vec4 b) { return v4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
SWH_HD inline Vec4 operator*(Vec4 a, float s) { return v4(a.x * s, a.y * s, a.z * s, a.w * s); }

// Plane: vec . p = dist (src/common/plane.rs)
struct Plane
{
	Vec3 vec;
	float dist;
};

// Column-major 4x4 matrix (cgmath Matrix4: c[0] is column x).
struct Mat4
{
	Vec4 c[4];
	SWH_HD static Mat4 identity()
	{
		Mat4 m;
		m.c[0] = v4(1, 0, 0, 0);
		m.c[1] = v4(0, 1, 0, 0);
		m.c[2] = v4(0, 0, 1, 0);
		m.c[3] = v4(0, 0, 0, 1);
		return m;
	}
	SWH_HD float at(int row, int col) const
	{
		const Vec4& v = c[col];
		return row == 0 ? v.x : row == 1 ? v.y : row == 2 ? v.z : v.w;
	}
	SWH_HD Vec4 row(int r) const { return v4(at(r, 0), at(r, 1), at(r, 2), at(r, 3)); }
};

// matrix * vector = c0*x + c1*y + c2*z + c3*w (left to right)
SWH_HD inline Vec4 operator*(const Mat4& m, Vec4 v) { return m.c[0] * v.x + m.c[1] * v.y + m.c[2] * v.z + m.c[3] * v.w; }
SWH_HD inline Mat4 operator*(const Mat4& a, const Mat4& b)
{
	Mat4 r;
	for (int i = 0; i < 4; ++i) r.c[i] = a * b.c[i];
	return r;
}
SWH_HD inline Mat4 transpose(const Mat4& m)
{
	Mat4 r;
	for (int i = 0; i < 4; ++i) r.c[i] = m.row(i);
	return r;
}

// Cofactor inverse; returns false for a singular matrix.
inline bool invert(const Mat4& m, Mat4& out)
{
	float a[16];
	for (int col = 0; col < 4; ++col)
		for (int row = 0; row < 4; ++row) a[col * 4 + row] = m.at(row, col);
	float inv[16];
	inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] -
		a[13] * a[7] * a[10];
	inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] +
		a[12] * a[7] * a[10];
	inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] -
		a[12] * a[7] * a[9];
	inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] +
		a[12] * a[6] * a[9];
	inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] +
		a[13] * a[3] * a[10];
	inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] -
		a[12] * a[3] * a[10];
	inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] +
		a[12] * a[3] * a[9];
	inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] -
		a[12] * a[2] * a[9];
	inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] -
		a[13] * a[3] * a[6];
	inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] +
		a[12] * a[3] * a[6];
	inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] -
		a[12] * a[3] * a[5];
	inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] +
		a[12] * a[2] * a[5];
	inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] +
		a[9] * a[3] * a[6];
	inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] -
		a[8] * a[3] * a[6];
	inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] +
		a[8] * a[3] * a[5];
	inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] -
		a[8] * a[2] * a[5];
	const float det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
	if (det == 0.0f || !std::isfinite(det)) return false;
	const float inv_det = 1.0f / det;
	for (int col = 0; col < 4; ++col)
		out.c[col] = v4(inv[col * 4 + 0] * inv_det, inv[col * 4 + 1] * inv_det, inv[col * 4 + 2] * inv_det, inv[col * 4 + 3] * inv_det);
	return true;
}

// Unit quaternion (cgmath Quaternion { s, v }).
struct Quat
{
	float s;
	Vec3 v;
};
inline Quat quat_mul(Quat a, Quat b)
{
	return Quat{a.s * b.s - a.v.x * b.v.x - a.v.y * b.v.y - a.v.z * b.v.z,
		v3(a.s * b.v.x + a.v.x * b.s + a.v.y * b.v.z - a.v.z * b.v.y, a.s * b.v.y + a.v.y * b.s + a.v.z * b.v.x - a.v.x * b.v.z,
			a.s * b.v.z + a.v.z * b.s + a.v.x * b.v.y - a.v.y * b.v.x)};
}
inline Quat quat_from_angle_z(float a) { return Quat{std::cos(a * 0.5f), v3(0, 0, std::sin(a * 0.5f))}; }
inline Quat quat_from_angle_y(float a) { return Quat{std::cos(a * 0.5f), v3(0, std::sin(a * 0.5f), 0)}; }
inline Quat conjugate(Quat q) { return Quat{q.s, -q.v}; }
// cgmath From<Quaternion> for Matrix4
inline Mat4 mat4_from_quat(Quat q)
{
	const float x2 = q.v.x + q.v.x, y2 = q.v.y + q.v.y, z2 = q.v.z + q.v.z;
	const float xx2 = x2 * q.v.x, xy2 = x2 * q.v.y, xz2 = x2 * q.v.z;
	const float yy2 = y2 * q.v.y, yz2 = y2 * q.v.z, zz2 = z2 * q.v.z;
	const float sy2 = y2 * q.s, sz2 = z2 * q.s, sx2 = x2 * q.s;
	Mat4 m;
	m.c[0] = v4(1.0f - yy2 - zz2, xy2 + sz2, xz2 - sy2, 0.0f);
	m.c[1] = v4(xy2 - sz2, 1.0f - xx2 - zz2, yz2 + sx2, 0.0f);
	m.c[2] = v4(xz2 + sy2, yz2 - sx2, 1.0f - xx2 - yy2, 0.0f);
	m.c[3] = v4(0, 0, 0, 1);
	return m;
}

// CameraMatrices, src/common/matrix.rs:3-11
struct CameraMatrices
{
	Vec3 position;
	Mat4 view_matrix;
	Mat4 planes_matrix;
};

// complete_view_matrix, src/common/matrix.rs:84-108: viewport shift * viewport scale * perspective *
// rotation * translation, and the planes matrix as the inverse of its transpose.
inline CameraMatrices complete_view_matrix(Vec3 position, const Mat4& rotation_matrix, Vec2 fov_scale, float width, float height)
{
	Mat4 translate = Mat4::identity();
	translate.c[3] = v4(-position.x, -position.y, -position.z, 1.0f);
	Mat4 perspective = Mat4::identity();
	perspective.c[0].x = fov_scale.x;
	perspective.c[1].y = fov_scale.y;
	Mat4 resize = Mat4::identity();
	resize.c[0].x = width * 0.5f;
	resize.c[1].y = height * 0.5f;
	Mat4 shift = Mat4::identity();
	shift.c[2].x = width * 0.5f;
	shift.c[2].y = height * 0.5f;

	CameraMatrices m;
	m.position = position;
	m.view_matrix = shift * resize * perspective * rotation_matrix * translate;
	Mat4 inv;
	if (!invert(transpose(m.view_matrix), inv)) inv = Mat4::identity();
	m.planes_matrix = inv;
	return m;
}

// build_view_matrix, src/common/matrix.rs:13-82
inline CameraMatrices build_view_matrix(Vec3 position, float azimuth, float elevation, float fov, float width, float height)
{
	const float pi = 3.14159265358979323846f;
	const Quat rotation = quat_mul(quat_from_angle_z(azimuth + pi * 0.5f), quat_from_angle_y(-elevation));
	const float inv_half_fov_tan = 1.0f / std::tan(fov * 0.5f);
	const float aspect = width / height;
	const Vec2 fov_scale = v2(inv_half_fov_tan / aspect, inv_half_fov_tan);

	Mat4 basis_change = Mat4::identity();
	basis_change.c[0] = v4(0, 0, 1, 0);
	basis_change.c[1] = v4(-1, 0, 0, 0);
	basis_change.c[2] = v4(0, -1, 0, 0);
	const Mat4 rotation_matrix = basis_change * mat4_from_quat(conjugate(rotation));
	return complete_view_matrix(position, rotation_matrix, fov_scale, width, height);
}

// build_view_matrix_with_full_rotation with get_full_ortation_matrix, src/common/matrix.rs:31-80 (used by
// calculate_projector_shadow_map_matrices, light.rs:63-71).
inline CameraMatrices build_view_matrix_with_full_rotation(Vec3 position, Quat rotation, float fov, float width, float height)
{
	const float inv_half_fov_tan = 1.0f / std::tan(fov * 0.5f);
	const float aspect = width / height;
	const Vec2 fov_scale = v2(inv_half_fov_tan / aspect, inv_half_fov_tan);
	Mat4 basis_change = Mat4::identity();
	basis_change.c[0] = v4(0, 0, 1, 0);
	basis_change.c[1] = v4(-1, 0, 0, 0);
	basis_change.c[2] = v4(0, -1, 0, 0);
	return complete_view_matrix(position, basis_change * mat4_from_quat(conjugate(rotation)), fov_scale, width, height);
}

// Quaternion::rotate_vector (through the rotation matrix).
inline Vec3 rotate_vector(Quat q, Vec3 v) { return truncate(mat4_from_quat(q) * extend(v, 0.0f)); }

// calculate_cube_shadow_map_side_matrices / get_cube_map_side_matrix, src/square_wheel/light.rs:73-133:
// side 0..5 = +X, -X, +Y, -Y, +Z, -Z; a 90-degree view (fov scale 1) over a size x size map.
inline CameraMatrices cube_shadow_map_side_matrices(Vec3 position, float size, uint32_t side)
{
	Mat4 m = Mat4::identity();
	const Vec4 ux = v4(1, 0, 0, 0), uy = v4(0, 1, 0, 0), uz = v4(0, 0, 1, 0);
	const Vec4 nx = v4(-1, 0, 0, 0), ny = v4(0, -1, 0, 0), nz = v4(0, 0, -1, 0);
	switch (side)
	{
	case 0: m.c[0] = uz, m.c[1] = nx, m.c[2] = ny; break;
	case 1: m.c[0] = nz, m.c[1] = ux, m.c[2] = ny; break;
	case 2: m.c[0] = ux, m.c[1] = uz, m.c[2] = ny; break;
	case 3: m.c[0] = nx, m.c[1] = nz, m.c[2] = ny; break;
	case 4: m.c[0] = ux, m.c[1] = uy, m.c[2] = uz; break;
	default: m.c[0] = ux, m.c[1] = ny, m.c[2] = nz; break;
	}
	return complete_view_matrix(position, m, v2(1.0f, 1.0f), size, size);
}

// view_matrix_transform_vertex, src/common/matrix.rs:125-128
SWH_HD inline Vec3 view_transform(const Mat4& m, Vec3 v) { return truncate(m * extend(v, 1.0f)); }

} // namespace swhost
