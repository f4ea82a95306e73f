/* Language features in one pixel shader: uniforms of three types, a
   function with an out parameter, loops with break, a switch, casts,
   write masks, swizzles, derivatives of inputs and intrinsics. */
float4 tint;
int    steps;
float  limit;

struct PSIn {
	float  v: TEXCOORD0;
	float3 n: TEXCOORD1;
	float4 q: TEXCOORD2;
};

struct PSOut {
	float4 c0: COLOR0;
	float4 c1: COLOR1;
	float2 c2: COLOR2;
	float3 c3: COLOR3;
};

float poly(float x, out float sq) {
	sq = x * x;
	return sq * x - 2.0f * x + 1.0f;
}

PSOut ps_main(PSIn in) {
	PSOut o;
	float sq;
	float p = poly(in.v, sq);
	float acc = in.v;
	for (int i = 0; i < steps; ++i) {
		acc = acc * 1.5f + 0.25f;
		if (acc > limit) { break; }
	}
	int k = 0;
	while (k < 3 && acc > 0.0f) {
		acc -= 1.0f;
		k++;
	}
	o.c0 = float4(p, sq, acc, (float)k) * tint;
	float3 c = cross(in.n, in.q.xyz);
	o.c1.xzy = normalize(c);
	o.c1.w = dot(in.n, in.q.xyz);
	o.c2 = ddx(in.q).yx + ddy(in.q.zw);
	o.c3 = (in.v > 0.5f) ? sqrt(abs(in.n)) : max(in.n, 0.25f).zyx;
	switch (k) {
	case 0: o.c3.x += 1.0f; break;
	case 1: o.c3.y += 2.0f; break;
	default: o.c3.z -= 3.0f;
	}
	return o;
}
