{
   /* Analytic spheres (rendered as UV spheres when the loader is asked to tessellate them): a
    * Phong sphere, a dielectric sphere, a named diffuse sphere and an instance of it, on a floor
    * under a unit-plane light. */
   "scenefile" : {
      "renderer" : { "type" : "pathTracer", "noSuperSamples" : 8, "noDirectSamples" : 2,
                     "maxDepth" : 5, "rrStartDepth" : 3, },
      "camera" : { "type" : "pinhole", "eye" : [ 0, 1.2, 4 ], "look" : [ 0, -0.2, -1 ], "up" : [ 0, 1, 0 ],
                   "heightAngle" : 40, },
      "output" : { "width" : 48, "height" : 36, },
      "scene" : {
         "material" : {
            "bsdf" : { "type" : "diffuse", "kd" : [ 0.6, 0.6, 0.55 ], },
            "plane" : { "vertices" : [ -3, 0, 3,   3, 0, 3,   3, 0, -3,   -3, 0, -3 ], },
         },
         "material" : {
            "bsdf" : { "type" : "phong", "kd" : 0.2, "ks" : 0.6, "n" : 60, },
            "sphere" : { "position" : [ -0.9, 0.45, 0 ], "radius" : 0.45, },
         },
         "material" : {
            "bsdf" : { "type" : "dielectric", "ior" : 1.5, },
            "transform" : {
               "translate" : [ 0.2, 0.5, 0.4 ],
               "sphere" : { "radius" : 0.5, },
            },
         },
         "material" : {
            "bsdf" : { "type" : "diffuse", "kd" : [ 0.2, 0.3, 0.7 ], },
            "sphere" : { "name" : "ball", "position" : [ 1.1, 0.3, -0.4 ], "radius" : 0.3, },
            "transform" : {
               "translate" : [ 0, 0, -1 ],
               "shape" : { "instance" : "ball" },
            },
         },
         "material" : {
            "emitter" : { "type" : "oriented", "power" : [ 24, 24, 20 ], },
            "transform" : {
               "translate" : [ 0, 2.5, 0 ],
               "rotate" : [ 0, 0, 0,  1, 0, 0,  180 ],
               "plane" : { },
            },
         },
      },
   },
}
